// adjoint.cu -- matched adjoints (exact transposes) of the ray-driven
// forward projectors, for gradients and for solvers that need A^T.
//
// Each kernel repeats its forward's ray set-up and sample points exactly and
// scatters y_ray * (filter weights) into the same pair-packed, zero-padded
// layouts the forward gathers from, with one 8-byte vector atomic per pair
// (red.global.add.v2.f32), or -- when the accumulators fit in L2 -- one
// 16-byte atomic per sample into quad accumulators.  A fold pass then adds the pair entries back onto
// the texels they cover; entries that land in the padding correspond to the
// zero border the forward reads and are dropped, so the result is the exact
// transpose of the forward as implemented.  The curadon reference has no
// matched adjoint (its backward of the forward is the voxel-driven
// backprojector, diffable.py:21-24); this is an addition beside it.
#include <cfloat>

#include "common.cuh"

namespace cg {
namespace {

// ------------------------------------------------------------ 2D

// QUAD: one float4 per (row, column) of the layout holding the contributions
// to (row, col), (row, col + 1), (row + 1, col), (row + 1, col + 1), so a
// sample is one 16-byte atomic instead of two 8-byte ones.
template <bool QUAD>
__device__ __forceinline__ void adj2d_ray(void *__restrict__ accA, void *__restrict__ accB,
                                          const float *__restrict__ sino,
                                          const float2 *__restrict__ tsrc,
                                          const float2 *__restrict__ tu0,
                                          const float2 *__restrict__ tdu, int W, int H, int det,
                                          int nangles, float sx, float sy, int pa, int pb, int u,
                                          int view) {
    if (u >= det || view >= nangles) return;
    const float2 s = tsrc[view], o = tu0[view], du = tdu[view];
    const float fu = (float)u;
    const float dx = fmaf(du.x, fu, o.x);
    const float dy = fmaf(du.y, fu, o.y);
    float tmin = FLT_MIN, tmax = FLT_MAX;
    {
        const float t1 = __fdividef(-1.f - s.x, dx), t2 = __fdividef((float)W - s.x, dx);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.y, dy), t2 = __fdividef((float)H - s.y, dy);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    if ((double)tmin > (double)tmax - 1e-6) return;
    const float rox = fmaf(dx, tmin, s.x), roy = fmaf(dy, tmin, s.y);
    const float tl = tmax - tmin;
    const float rdx = dx * tl, rdy = dy * tl;
    const float m = fmaxf(fabsf(rdx), fabsf(rdy));
    int n = __float2int_rn(m);
    const float vx = rdx / m, vy = rdy / m;
    const float c = sino[(size_t)view * det + u] * hypotf(vx * sx, vy * sy);
    if (c == 0.f) return;

    const bool ymajor = fabsf(rdy) >= fabsf(rdx);
    float p = (ymajor ? rox : roy) - 0.5f;
    const float vp = ymajor ? vx : vy;
    const float q = (ymajor ? roy : rox) - 0.5f;
    const int sq = ((ymajor ? vy : vx) > 0.f) ? 1 : -1;
    void *acc = ymajor ? accA : accB;
    const int pitch = ymajor ? pa : pb;
    const float pmax = (float)(ymajor ? W : H);
    const int qmax = ymajor ? H : W;
    const float qf = floorf(q);
    const float fq = q - qf;
    const int iq = (int)fminf(fmaxf(qf, -(float)kPad), (float)qmax);
    n = min(n, sq > 0 ? qmax - iq + 1 : iq + kPad + 1);
    long long ri = (long long)(iq + kPad) * pitch + kPad;  // element of the row start
    const long long rstep = (long long)sq * pitch;
    const float clo = c * (1.f - fq), chi = c * fq;
    for (int j = 0; j < n; ++j) {
        const float pf = fminf(fmaxf(floorf(p), -(float)kPad), pmax);
        const float fp = p - pf;
        const int ip = (int)pf;
        // forward: lo = x + fp (y - x) -> weights (1 - fp, fp) on the pair
        if constexpr (QUAD) {
            atomicAdd(static_cast<float4 *>(acc) + ri + ip,
                      make_float4(clo * (1.f - fp), clo * fp, chi * (1.f - fp), chi * fp));
        } else {
            float2 *row = static_cast<float2 *>(acc) + ri;
            atomicAdd(row + ip, make_float2(clo * (1.f - fp), clo * fp));
            atomicAdd(row + pitch + ip, make_float2(chi * (1.f - fp), chi * fp));
        }
        p += vp;
        ri += rstep;
    }
}

template <bool QUAD>
__global__ void __launch_bounds__(256)
    k_adj2d(void *__restrict__ accA, void *__restrict__ accB, const float *__restrict__ sino,
            const float2 *__restrict__ tsrc, const float2 *__restrict__ tu0,
            const float2 *__restrict__ tdu, int W, int H, int det, int nangles, float sx,
            float sy, int pa, int pb) {
    adj2d_ray<QUAD>(accA, accB, sino, tsrc, tu0, tdu, W, H, det, nangles, sx, sy, pa, pb,
                    blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

// vol[y][x] += the four quad entries covering (x, y) in each layout.
__device__ __forceinline__ void fold2d_quad(float *__restrict__ vol, const float4 *__restrict__ A,
                                            const float4 *__restrict__ B, int W, int H, int pa,
                                            int pb, int x, int y) {
    if (x >= W || y >= H) return;
    const float4 *ra = A + (size_t)(y + kPad) * pa + (x + kPad);
    const float4 *rb = B + (size_t)(x + kPad) * pb + (y + kPad);
    const float sa = (ra[0].x + ra[-1].y) + (ra[-pa].z + ra[-pa - 1].w);
    const float sb = (rb[0].x + rb[-1].y) + (rb[-pb].z + rb[-pb - 1].w);
    vol[(size_t)y * W + x] += sa + sb;
}

__global__ void k_fold2d_quad(float *__restrict__ vol, const float4 *__restrict__ A,
                              const float4 *__restrict__ B, int W, int H, int pa, int pb) {
    fold2d_quad(vol, A, B, W, H, pa, pb, blockIdx.x * blockDim.x + threadIdx.x,
                blockIdx.y * blockDim.y + threadIdx.y);
}

// The matched adjoint of a batch (quad accumulators), as three launches over
// the batch's work list: zeroing every problem's accumulators, the scatter
// (one ray per thread, 32 cells x 8 views per block) and the fold (one voxel
// per thread, 32 x 8 per block).  Each problem's result equals its
// single-problem matched adjoint up to the order of the atomic additions.
__global__ void __launch_bounds__(256)
    k_batch_adj2d_zero(const Prob2d *__restrict__ probs, const int *__restrict__ start,
                       int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const long long na = (long long)q.pa * (q.H + 2 * kPad);
    const long long nb = (long long)q.pb * (q.W + 2 * kPad);
    const long long base = (long long)(blockIdx.x - start[i]) * 1024;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const long long e = base + k * 256 + threadIdx.x;
        if (e < na) q.quadA[e] = z;
        else if (e < na + nb) q.quadB[e - na] = z;
    }
}

__global__ void __launch_bounds__(256)
    k_batch_adj2d(const Prob2d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.det + 31) / 32;
    adj2d_ray<true>(q.quadA, q.quadB, q.sino, q.src, q.u0, q.du, q.W, q.H, q.det, q.nangles, q.sx,
                    q.sy, q.pa, q.pb, (local % gx) * 32 + threadIdx.x,
                    (local / gx) * 8 + threadIdx.y);
}

__global__ void __launch_bounds__(256)
    k_batch_fold2d(const Prob2d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.W + 31) / 32;
    fold2d_quad(q.vol, q.quadA, q.quadB, q.W, q.H, q.pa, q.pb, (local % gx) * 32 + threadIdx.x,
                (local / gx) * 8 + threadIdx.y);
}

// vol[y][x] += A[y][x].x + A[y][x-1].y + B[x][y].x + B[x][y-1].y (padded).
__global__ void k_fold2d(float *__restrict__ vol, const float2 *__restrict__ A,
                         const float2 *__restrict__ B, int W, int H, int pa, int pb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float2 *ra = A + (size_t)(y + kPad) * pa + kPad;
    const float2 *rb = B + (size_t)(x + kPad) * pb + kPad;
    vol[(size_t)y * W + x] += (ra[x].x + ra[x - 1].y) + (rb[y].x + rb[y - 1].y);
}

// ------------------------------------------------------------ 3D

// QUAD: the accumulators hold, per (a, b, c), the four contributions to
// voxels (a, b), (a + 1, b), (a, b + 1), (a + 1, b + 1) of slice c as one
// float4, so a sample is two 16-byte atomics instead of four 8-byte ones
// (the scatter is bound by the L2's atomic operations).
// BAND: blocks of 32 x 8 cells of one view in a linear grid ordered cells,
// then views, then bands of 8 detector rows, each warp on an 8 x 4 patch of
// cells (the quad forward's order): the blocks resident at one time scatter
// into a slab of the volume's y range, so the atomics stay in L2; otherwise
// a (U/32, V/8, views) grid of 32 x 8 blocks.
// MERGE (quads): a sample's upper-slice contribution is held in registers
// and, when the next sample's lower slice is the same element (the ray
// advanced one slice within the same row and column), added to it, so the
// two go out as one atomic.
// AGG (quads, with MERGE): warp-aggregated atomics -- the lanes of a warp
// whose lower-slice element coincides at a step (found with
// __match_any_sync) pass their contributions through shared memory to the
// lowest such lane, which sums them in lane order and issues one atomic.
// The band-major block `lin`'s cell of this thread.
__device__ __forceinline__ void adj3d_band_cell(int lin, int utiles, int P, int &iu, int &iv,
                                                int &view) {
    const int ut = lin % utiles, rest = lin / utiles;
    view = rest % P;
    const int band = rest / P;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    iu = ut * 32 + (warp & 3) * 8 + (lane & 7);
    iv = band * 8 + (warp >> 2) * 4 + (lane >> 3);
}

// One ray's scatter (the cell (iu, iv) of `view`).
template <bool QUAD, bool MERGE, bool AGG>
__device__ __forceinline__ void adj3d_ray(void *__restrict__ A, void *__restrict__ B,
                                          const float *__restrict__ sino,
                                          const float4 *__restrict__ torg,
                                          const float4 *__restrict__ tdu,
                                          const float4 *__restrict__ tdv,
                                          const float4 *__restrict__ tsrc, int X, int Y, int Z,
                                          int U, int V, bool exact_t, int iu, int iv, int view) {
    if (iu >= U || iv >= V) return;
    const float c = sino[((size_t)view * V + iv) * U + iu];
    if (c == 0.f) return;
    const float4 o = torg[view], du = tdu[view], dv = tdv[view], s = tsrc[view];
    const float fu = (float)iu, fv = (float)iv;
    const float detx = o.x + fu * du.x + fv * dv.x;
    const float dety = o.y + fu * du.y + fv * dv.y;
    const float detz = o.z + fu * du.z + fv * dv.z;
    const float dx = detx - s.x, dy = dety - s.y, dz = detz - s.z;
    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
    const long long nsamples = (long long)ceilf(__fdividef(len, 1.0f));
    float tmin = FLT_MIN, tmax = FLT_MAX;
    {
        const float t1 = __fdividef(-1.f - s.x, dx), t2 = __fdividef((float)(X + 1) - s.x, dx);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.y, dy), t2 = __fdividef((float)(Y + 1) - s.y, dy);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.z, dz), t2 = __fdividef((float)(Z + 1) - s.z, dz);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    if (!(tmin <= tmax)) return;
    const int nsteps = (int)ceilf((tmax - tmin) * (float)nsamples);
    const float h = (tmax - tmin) / (float)nsteps;
    if (!(h > 0.f) || !isfinite(tmax) || nsteps > (1 << 22)) return;

    const bool xmajor = fabsf(dx) > fabsf(dz);
    const float sa = xmajor ? s.z : s.x, da = xmajor ? dz : dx;
    const float sc = xmajor ? s.x : s.z, dc = xmajor ? dx : dz;
    void *L = xmajor ? B : A;
    const int Na = xmajor ? Z : X, Nc = xmajor ? X : Z;
    const int pa = Na + 2 * kPad, pb = Y + 2 * kPad;
    const float amax = (float)Na, bmax = (float)Y, cmax = (float)Nc;
    const float lo = -(float)kPad;
    float t = tmin;
    size_t held_at = ~(size_t)0;  // MERGE: element of the held contribution
    float4 held = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k <= nsteps + 1; ++k) {
        if (!(t <= tmax)) break;
        const float pa_ = fmaf(da, t, sa), pb_ = fmaf(dy, t, s.y), pc_ = fmaf(dc, t, sc);
        const float fa = fminf(fmaxf(floorf(pa_), lo), amax);
        const float fb = fminf(fmaxf(floorf(pb_), lo), bmax);
        const float fc = fminf(fmaxf(floorf(pc_), lo), cmax);
        const float wa = pa_ - fa, wb = pb_ - fb, wc = pc_ - fc;
        const size_t i00 = ((size_t)((int)fc + kPad) * pb + ((int)fb + kPad)) * pa + ((int)fa + kPad);
        const float c00 = c * (1.f - wb) * (1.f - wc), c10 = c * wb * (1.f - wc);
        const float c01 = c * (1.f - wb) * wc, c11 = c * wb * wc;
        if constexpr (QUAD && MERGE) {
            float4 *q = static_cast<float4 *>(L);
            float4 lower = make_float4(c00 * (1.f - wa), c00 * wa, c10 * (1.f - wa), c10 * wa);
            const float4 upper =
                make_float4(c01 * (1.f - wa), c01 * wa, c11 * (1.f - wa), c11 * wa);
            if (i00 == held_at) {
                lower.x += held.x, lower.y += held.y, lower.z += held.z, lower.w += held.w;
            } else if (held_at != ~(size_t)0) {
                atomicAdd(q + held_at, held);
            }
            if constexpr (AGG) {
                __shared__ float4 s_agg[8][32];
                const unsigned active = __activemask();
                const int lane = (int)(threadIdx.x + threadIdx.y * blockDim.x) & 31;
                const int wslot = (int)(threadIdx.x + threadIdx.y * blockDim.x) >> 5;
                const unsigned peers = __match_any_sync(active, (unsigned)i00);
                const int leader = __ffs(peers) - 1;
                // lanes that share their element with another lane; only
                // they take part in the exchange and its two warp barriers
                const unsigned shared = __ballot_sync(active, peers != (1u << lane));
                if (peers != (1u << lane)) {
                    if (lane != leader) s_agg[wslot][lane] = lower;
                    __syncwarp(shared);
                    if (lane == leader) {
                        for (unsigned rest = peers & ~(1u << lane); rest; rest &= rest - 1) {
                            const float4 o = s_agg[wslot][__ffs(rest) - 1];
                            lower.x += o.x, lower.y += o.y, lower.z += o.z, lower.w += o.w;
                        }
                    }
                    __syncwarp(shared);
                }
                if (lane == leader) atomicAdd(q + i00, lower);
            } else {
                atomicAdd(q + i00, lower);
            }
            held = upper, held_at = i00 + (size_t)pa * pb;
        } else if constexpr (QUAD) {
            float4 *q = static_cast<float4 *>(L) + i00;
            atomicAdd(q, make_float4(c00 * (1.f - wa), c00 * wa, c10 * (1.f - wa), c10 * wa));
            atomicAdd(q + (size_t)pa * pb,
                      make_float4(c01 * (1.f - wa), c01 * wa, c11 * (1.f - wa), c11 * wa));
        } else {
            float2 *p00 = static_cast<float2 *>(L) + i00;
            atomicAdd(p00, make_float2(c00 * (1.f - wa), c00 * wa));
            atomicAdd(p00 + pa, make_float2(c10 * (1.f - wa), c10 * wa));
            atomicAdd(p00 + (size_t)pa * pb, make_float2(c01 * (1.f - wa), c01 * wa));
            atomicAdd(p00 + (size_t)pa * pb + pa, make_float2(c11 * (1.f - wa), c11 * wa));
        }
        t = march_next(t, k, tmin, h, exact_t);
    }
    if constexpr (QUAD && MERGE) {
        if (held_at != ~(size_t)0) atomicAdd(static_cast<float4 *>(L) + held_at, held);
    }
}

template <bool QUAD, bool BAND = false, bool MERGE = false, bool AGG = false>
__global__ void __launch_bounds__(256)
    k_adj3d(void *__restrict__ A, void *__restrict__ B, const float *__restrict__ sino,
            const float4 *__restrict__ torg, const float4 *__restrict__ tdu,
            const float4 *__restrict__ tdv, const float4 *__restrict__ tsrc, int X, int Y, int Z,
            int U, int V, int P, int utiles, bool exact_t) {
    int iu, iv, view;
    if constexpr (BAND) {
        adj3d_band_cell(blockIdx.x, utiles, P, iu, iv, view);
    } else {
        iu = blockIdx.x * blockDim.x + threadIdx.x;
        iv = blockIdx.y * blockDim.y + threadIdx.y;
        view = blockIdx.z;
    }
    adj3d_ray<QUAD, MERGE, AGG>(A, B, sino, torg, tdu, tdv, tsrc, X, Y, Z, U, V, exact_t, iu, iv,
                                view);
}

// vol[z][y][x] += A[z][y][x].x + A[z][y][x-1].y + B[x][y][z].x + B[x][y][z-1].y
__global__ void k_fold3d(float *__restrict__ vol, const float2 *__restrict__ A,
                         const float2 *__restrict__ B, int X, int Y, int Z) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)X * Y * Z) return;
    const int x = (int)(idx % X);
    const int y = (int)((idx / X) % Y);
    const int z = (int)(idx / ((long long)X * Y));
    const int PX = X + 2 * kPad, PY = Y + 2 * kPad, PZ = Z + 2 * kPad;
    const float2 *ra = A + ((size_t)(z + kPad) * PY + (y + kPad)) * PX + (x + kPad);
    const float2 *rb = B + ((size_t)(x + kPad) * PY + (y + kPad)) * PZ + (z + kPad);
    vol[idx] += (ra[0].x + ra[-1].y) + (rb[0].x + rb[-1].y);
}

// The same fold for the quad accumulators: voxel (a, b) of slice c gathers
// .x of (a, b), .y of (a - 1, b), .z of (a, b - 1) and .w of (a - 1, b - 1).
__device__ __forceinline__ void fold3d_quad_at(float *__restrict__ vol,
                                               const float4 *__restrict__ A,
                                               const float4 *__restrict__ B, int X, int Y, int Z,
                                               long long idx) {
    if (idx >= (long long)X * Y * Z) return;
    const int x = (int)(idx % X);
    const int y = (int)((idx / X) % Y);
    const int z = (int)(idx / ((long long)X * Y));
    const int PX = X + 2 * kPad, PY = Y + 2 * kPad, PZ = Z + 2 * kPad;
    const float4 *ra = A + ((size_t)(z + kPad) * PY + (y + kPad)) * PX + (x + kPad);
    const float4 *rb = B + ((size_t)(x + kPad) * PY + (y + kPad)) * PZ + (z + kPad);
    const float sa = (ra[0].x + ra[-1].y) + (ra[-PX].z + ra[-PX - 1].w);
    const float sb = (rb[0].x + rb[-1].y) + (rb[-PZ].z + rb[-PZ - 1].w);
    vol[idx] += sa + sb;
}

__global__ void k_fold3d_quad(float *__restrict__ vol, const float4 *__restrict__ A,
                              const float4 *__restrict__ B, int X, int Y, int Z) {
    fold3d_quad_at(vol, A, B, X, Y, Z, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---- 3D batches: the matched adjoint of every problem over one work list
// (the quad accumulators zeroed, the merged quad scatter in band-major
// order, the fold), the transpose partner of the batched quad forward
// without texture warps.

__global__ void __launch_bounds__(256)
    k_batch_adj3d_zero(const Prob3d *__restrict__ probs, const int *__restrict__ start,
                       int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    const long long idx = (long long)(blockIdx.x - start[i]) * blockDim.x + threadIdx.x;
    const long long n = (long long)(q.X + 2 * kPad) * (q.Y + 2 * kPad) * (q.Z + 2 * kPad);
    if (idx < n) q.adjA[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
    else if (idx < 2 * n) q.adjB[idx - n] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void __launch_bounds__(256)
    k_batch_adj3d(const Prob3d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    int iu, iv, view;
    adj3d_band_cell(blockIdx.x - start[i], q.utiles, q.P, iu, iv, view);
    adj3d_ray<true, true, false>(q.adjA, q.adjB, q.sino, q.forg, q.fdu, q.fdv, q.fsrc, q.X, q.Y,
                                 q.Z, q.U, q.V, q.exact_t != 0, iu, iv, view);
}

__global__ void __launch_bounds__(256)
    k_batch_fold3d(const Prob3d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    fold3d_quad_at(q.vol, q.adjA, q.adjB, q.X, q.Y, q.Z,
                   (long long)(blockIdx.x - start[i]) * blockDim.x + threadIdx.x);
}

}  // namespace

size_t adj2d_quad_elems(const Plan2d &p, bool layoutA) {
    return layoutA ? (size_t)p.pitchA() * (p.H + 2 * kPad) : (size_t)p.pitchB() * (p.W + 2 * kPad);
}

int ensure_adj2d_quads(Plan2d &p) {
    if (p.d_quadA) return CG_OK;
    CG_TRY_CUDA(cudaMalloc(&p.d_quadA, adj2d_quad_elems(p, true) * sizeof(float4)));
    CG_TRY_CUDA(cudaMalloc(&p.d_quadB, adj2d_quad_elems(p, false) * sizeof(float4)));
    return CG_OK;
}

int launch_batch2d_adjoint(const Prob2d *probs, const int *starts,
                           const int totals[kBatchStages], int count, cudaStream_t s) {
    const dim3 tile(32, 8);
    k_batch_adj2d_zero<<<totals[4], 256, 0, s>>>(probs, starts + 4 * (count + 1), count);
    CG_TRY_CUDA(cudaGetLastError());
    k_batch_adj2d<<<totals[5], tile, 0, s>>>(probs, starts + 5 * (count + 1), count);
    CG_TRY_CUDA(cudaGetLastError());
    k_batch_fold2d<<<totals[6], tile, 0, s>>>(probs, starts + 6 * (count + 1), count);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_adjoint2d(Plan2d &p, float *vol, const float *sino, cudaStream_t s) {
    const size_t na = adj2d_quad_elems(p, true);
    const size_t nb = adj2d_quad_elems(p, false);
    dim3 block(p.fwd_bx, p.fwd_by);
    dim3 grid(ceil_div(p.det, p.fwd_bx), ceil_div(p.nangles, p.fwd_by));
    if (grid.y > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    const dim3 fgrid(ceil_div(p.W, 32), ceil_div(p.H, 8));
    // quad accumulators when both fit in 96 MB, where the L2 holds the atomics
    if (p.adj_quad > 0 || (p.adj_quad < 0 && (na + nb) * sizeof(float4) <= (96u << 20))) {
        if (int rc = ensure_adj2d_quads(p)) return rc;
        CG_TRY_CUDA(cudaMemsetAsync(p.d_quadA, 0, na * sizeof(float4), s));
        CG_TRY_CUDA(cudaMemsetAsync(p.d_quadB, 0, nb * sizeof(float4), s));
        k_adj2d<true><<<grid, block, 0, s>>>(p.d_quadA, p.d_quadB, sino, p.d_src, p.d_u0, p.d_du,
                                             p.W, p.H, p.det, p.nangles, p.sx, p.sy, p.pitchA(),
                                             p.pitchB());
        CG_TRY_CUDA(cudaGetLastError());
        k_fold2d_quad<<<fgrid, dim3(32, 8), 0, s>>>(vol, p.d_quadA, p.d_quadB, p.W, p.H,
                                                    p.pitchA(), p.pitchB());
        CG_TRY_CUDA(cudaGetLastError());
        return CG_OK;
    }
    CG_TRY_CUDA(cudaMemsetAsync(p.d_layA, 0, na * sizeof(float2), s));
    CG_TRY_CUDA(cudaMemsetAsync(p.d_layB, 0, nb * sizeof(float2), s));
    k_adj2d<false><<<grid, block, 0, s>>>(p.d_layA, p.d_layB, sino, p.d_src, p.d_u0, p.d_du, p.W,
                                          p.H, p.det, p.nangles, p.sx, p.sy, p.pitchA(),
                                          p.pitchB());
    CG_TRY_CUDA(cudaGetLastError());
    k_fold2d<<<fgrid, dim3(32, 8), 0, s>>>(vol, p.d_layA, p.d_layB, p.W, p.H, p.pitchA(),
                                           p.pitchB());
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int ensure_adj3d_quads(Plan3d &p) {
    if (p.d_quadA) return CG_OK;
    const size_t elems = (size_t)(p.X + 2 * kPad) * (p.Y + 2 * kPad) * (p.Z + 2 * kPad);
    CG_TRY_CUDA(cudaMalloc(&p.d_quadA, elems * sizeof(float4)));
    if (cudaMalloc(&p.d_quadB, elems * sizeof(float4)) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaFree(p.d_quadA);
        p.d_quadA = nullptr;
        return set_error(CG_ERR_NOMEM, "no room for the matched adjoint's accumulators");
    }
    return CG_OK;
}

int launch_batch3d_adjoint(const Prob3d *d_probs, const int *starts,
                           const int totals[kBatch3dStages], int count, cudaStream_t s) {
    const int n1 = count + 1;
    if (totals[6] > 0) {
        k_batch_adj3d_zero<<<totals[6], 256, 0, s>>>(d_probs, starts + 6 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (totals[7] > 0) {
        k_batch_adj3d<<<totals[7], dim3(32, 8), 0, s>>>(d_probs, starts + 7 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (totals[8] > 0) {
        k_batch_fold3d<<<totals[8], 256, 0, s>>>(d_probs, starts + 8 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    return CG_OK;
}

int launch_adjoint3d(Plan3d &p, float *vol, const float *sino, cudaStream_t s) {
    if (p.nangles > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    const int utiles = ceil_div(p.U, 32);
    const long long bblocks = (long long)utiles * p.nangles * ceil_div(p.V, 8);
    const long long n = (long long)p.X * p.Y * p.Z;
    const size_t elems = (size_t)(p.X + 2 * kPad) * (p.Y + 2 * kPad) * (p.Z + 2 * kPad);
    // measured at 128^3 (74 MB of quad accumulators, L2-resident) and 256^3
    // (281 MB): quads beat pairs at both (3.29 against 4.78 ms; 32.8 against
    // 47.2 ms); view-major order is best while the accumulators fit in L2,
    // band-major order (a y-slab of the volume at a time) once they do not
    // (256^3: 32.8 against 48.3 ms; 128^3: 3.64 against 3.29 ms)
    const bool quad = p.adj_quad != 0;
    const bool fits = 2 * elems * (quad ? sizeof(float4) : sizeof(float2)) <= (96u << 20);
    const bool band = (p.adj_band > 0 || (p.adj_band < 0 && !fits)) && bblocks < (1ll << 31);
    dim3 grid = band ? dim3((unsigned)bblocks) : dim3(utiles, ceil_div(p.V, 8), p.nangles);
    if (quad) {
        if (int rc = ensure_adj3d_quads(p)) return rc;
        CG_TRY_CUDA(cudaMemsetAsync(p.d_quadA, 0, elems * sizeof(float4), s));
        CG_TRY_CUDA(cudaMemsetAsync(p.d_quadB, 0, elems * sizeof(float4), s));
        auto kq = p.adj_agg   ? (band ? k_adj3d<true, true, true, true>
                                      : k_adj3d<true, false, true, true>)
                  : p.adj_merge ? (band ? k_adj3d<true, true, true> : k_adj3d<true, false, true>)
                                : (band ? k_adj3d<true, true> : k_adj3d<true, false>);
        kq<<<grid, dim3(32, 8), 0, s>>>(p.d_quadA, p.d_quadB, sino, p.d_forg, p.d_fdu, p.d_fdv,
                                        p.d_fsrc, p.X, p.Y, p.Z, p.U, p.V, p.nangles, utiles,
                                        p.exact_t);
        CG_TRY_CUDA(cudaGetLastError());
        k_fold3d_quad<<<ceil_div(n, 256), 256, 0, s>>>(vol, p.d_quadA, p.d_quadB, p.X, p.Y, p.Z);
        CG_TRY_CUDA(cudaGetLastError());
        return CG_OK;
    }
    CG_TRY_CUDA(cudaMemsetAsync(p.d_volA, 0, p.volA_elems * sizeof(float2), s));
    CG_TRY_CUDA(cudaMemsetAsync(p.d_volB, 0, p.volB_elems * sizeof(float2), s));
    auto kp = band ? k_adj3d<false, true> : k_adj3d<false, false>;
    kp<<<grid, dim3(32, 8), 0, s>>>(p.d_volA, p.d_volB, sino, p.d_forg, p.d_fdu, p.d_fdv,
                                    p.d_fsrc, p.X, p.Y, p.Z, p.U, p.V, p.nangles, utiles,
                                    p.exact_t);
    CG_TRY_CUDA(cudaGetLastError());
    k_fold3d<<<ceil_div(n, 256), 256, 0, s>>>(vol, p.d_volA, p.d_volB, p.X, p.Y, p.Z);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
