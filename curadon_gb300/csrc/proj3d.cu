// proj3d.cu -- 3D cone-beam projection kernels for sm_103a.
//
// Data layout in HBM (all float32, per plan, allocated on first use):
//   volA  (Z+2P)(Y+2P)(X+2P) float2, pairs along x: (v[z][y][x], v[z][y][x+1] - v[z][y][x])
//   volB  (X+2P)(Y+2P)(Z+2P) float2, pairs along z: (v[z][y][x], v[z+1][y][x] - v[z][y][x])
//   sinoP nangles (V+2P)(U+2P) float2, pairs along u as (s[u], s[u+1] - s[u])
// with P = kPad zero texels on every face.  A warp handles 32 adjacent
// detector cells; for a circular orbit about y those cells are spread along
// x when the ray runs along z and along z when it runs along x, so each ray
// samples the copy whose contiguous axis is the one its warp spreads over,
// and four 8-byte loads gather the eight texels of a trilinear sample.
#include <cfloat>
#include <climits>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace cg {
namespace {

constexpr int kP3 = kPad;
constexpr int kQP = 2 * kP3 + 1;  // quad copies: kP3 zero planes below, kP3 + 1 above

// ------------------------------------------------------------ re-layouts

__global__ void k_relayout3d_A(const float *__restrict__ vol, int X, int Y, int Z,
                               float2 *__restrict__ A) {
    const int PX = X + 2 * kP3, PY = Y + 2 * kP3, PZ = Z + 2 * kP3;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)PX * PY * PZ) return;
    const int a = (int)(idx % PX) - kP3;
    const long long r = idx / PX;
    const int b = (int)(r % PY) - kP3;
    const int c = (int)(r / PY) - kP3;
    float t0 = 0.f, t1 = 0.f;
    if (b >= 0 && b < Y && c >= 0 && c < Z) {
        const float *row = vol + ((size_t)c * Y + b) * X;
        if (a >= 0 && a < X) t0 = row[a];
        if (a + 1 >= 0 && a + 1 < X) t1 = row[a + 1];
    }
    A[idx] = make_float2(t0, t1 - t0);
}

// x <-> z transpose of one y plane, 32 x 32 tiles through shared memory.
__global__ void __launch_bounds__(256)
    k_relayout3d_B(const float *__restrict__ vol, int X, int Y, int Z, float2 *__restrict__ B) {
    __shared__ float tile[33][33];  // [z][x]
    const int PY = Y + 2 * kP3, PZ = Z + 2 * kP3, PX = X + 2 * kP3;
    const int x0 = blockIdx.x * 32 - kP3, z0 = blockIdx.y * 32 - kP3;
    const int b = (int)blockIdx.z - kP3;  // y
    const bool yin = b >= 0 && b < Y;
    for (int j = threadIdx.y; j < 33; j += blockDim.y)
        for (int i = threadIdx.x; i < 33; i += blockDim.x) {
            const int x = x0 + i, z = z0 + j;
            tile[j][i] = (yin && x >= 0 && x < X && z >= 0 && z < Z)
                             ? vol[((size_t)z * Y + b) * X + x]
                             : 0.f;
        }
    __syncthreads();
    const int tz = threadIdx.x;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int x = x0 + i, z = z0 + tz;
        if (x < X + kP3 && z < Z + kP3)
            B[((size_t)(x + kP3) * PY + (b + kP3)) * PZ + (z + kP3)] =
                make_float2(tile[tz][i], tile[tz + 1][i] - tile[tz][i]);
    }
    (void)PX;
}

// Quads of the volume for k_fwd3d_quad.  Element (c, b, a) holds, in slice
// c, the values at rows b, b + 1 and columns a, a + 1 as A = v00,
// B = v01 - v00, C = v10 - v00, D = (v11 - v10) - (v01 - v00) (first index
// the row), so the bilinear value at fractions (wa, wb) is
// A + wa B + wb (C + wa D).  Every axis is padded with kP3 zero planes below
// and kP3 + 1 above (kQP in all), so the samples of a ray inside the box
// [-1, N + 1]^3 and their slice c + 1 stay inside the array.
// QA: slices z, rows y, columns x.
__device__ __forceinline__ void relayout3d_qa_at(const float *__restrict__ vol, int X, int Y,
                                                 int Z, float4 *__restrict__ QA, long long idx) {
    const int PX = X + kQP, PY = Y + kQP, PZ = Z + kQP;
    if (idx >= (long long)PX * PY * PZ) return;
    const int x = (int)(idx % PX) - kP3;
    const long long r = idx / PX;
    const int y = (int)(r % PY) - kP3;
    const int z = (int)(r / PY) - kP3;
    float v[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    if (z >= 0 && z < Z)
        for (int i = 0; i < 2; ++i) {
            if (y + i < 0 || y + i >= Y) continue;
            const float *row = vol + ((size_t)z * Y + (y + i)) * X;
            if (x >= 0 && x < X) v[i][0] = row[x];
            if (x + 1 >= 0 && x + 1 < X) v[i][1] = row[x + 1];
        }
    const float b = v[0][1] - v[0][0];
    QA[idx] = make_float4(v[0][0], b, v[1][0] - v[0][0], (v[1][1] - v[1][0]) - b);
}

__global__ void k_relayout3d_qa(const float *__restrict__ vol, int X, int Y, int Z,
                                float4 *__restrict__ QA) {
    relayout3d_qa_at(vol, X, Y, Z, QA, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// QB: slices x, rows y, columns z; an x <-> z transpose of the rows y, y + 1
// through shared memory, 32 x 32 (x, z) tiles.
// One 32 x 32 (z, x) tile (ta, tc) of row b; a block of 32 x 8 threads.
__device__ __forceinline__ void relayout3d_qb_tile(const float *__restrict__ vol, int X, int Y,
                                                   int Z, float4 *__restrict__ QB, int ta, int tc,
                                                   int b) {
    __shared__ float tile[2][33][33];  // [row][z][x]
    const int PX = X + kQP, PY = Y + kQP, PZ = Z + kQP;
    const int a0 = ta * 32, c0 = tc * 32;
    const int z0 = a0 - kP3, x0 = c0 - kP3, y = b - kP3;
    for (int j = threadIdx.y; j < 33; j += blockDim.y)
        for (int i = 0; i < 2; ++i) {
            const int x = x0 + threadIdx.x, z = z0 + j, yy = y + i;
            tile[i][j][threadIdx.x] = (x >= 0 && x < X && z >= 0 && z < Z && yy >= 0 && yy < Y)
                                          ? vol[((size_t)z * Y + yy) * X + x]
                                          : 0.f;
        }
    __syncthreads();
    const int tz = threadIdx.x, a = a0 + tz;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i;
        if (c >= PX || a >= PZ) continue;
        const float v00 = tile[0][tz][i], v01 = tile[0][tz + 1][i];
        const float v10 = tile[1][tz][i], v11 = tile[1][tz + 1][i];
        const float bb = v01 - v00;
        QB[((size_t)c * PY + b) * PZ + a] = make_float4(v00, bb, v10 - v00, (v11 - v10) - bb);
    }
}

__global__ void __launch_bounds__(256)
    k_relayout3d_qb(const float *__restrict__ vol, int X, int Y, int Z, float4 *__restrict__ QB) {
    relayout3d_qb_tile(vol, X, Y, Z, QB, blockIdx.x, blockIdx.y, blockIdx.z);
}


__global__ void k_relayout_sino3d(const float *__restrict__ sino, int U, int V, int nangles,
                                  float2 *__restrict__ S) {
    const int PU = U + 2 * kP3, PV = V + 2 * kP3;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)PU * PV * nangles) return;
    const int a = (int)(idx % PU) - kP3;
    const long long r = idx / PU;
    const int b = (int)(r % PV) - kP3;
    const int view = (int)(r / PV);
    float t0 = 0.f, t1 = 0.f;
    if (b >= 0 && b < V) {
        const float *row = sino + ((size_t)view * V + b) * U;
        if (a >= 0 && a < U) t0 = row[a];
        if (a + 1 >= 0 && a + 1 < U) t1 = row[a + 1];
    }
    S[idx] = make_float2(t0, t1 - t0);
}

// The same layout with rows b and b + 1 in one float4 (pair of row b, pair
// of row b + 1), so a bilinear sample is one 16-byte load.
__device__ __forceinline__ void relayout_sino3d_quad_at(const float *__restrict__ sino, int U, int V,
                                                   int nangles, float4 *__restrict__ S,
                                                   long long idx) {
    const int PU = U + 2 * kP3, PV = V + 2 * kP3;
    if (idx >= (long long)PU * PV * nangles) return;
    const int a = (int)(idx % PU) - kP3;
    const long long r = idx / PU;
    const int b = (int)(r % PV) - kP3;
    const int view = (int)(r / PV);
    float t[4] = {0.f, 0.f, 0.f, 0.f};  // (row b: a, a + 1), (row b + 1: a, a + 1)
    for (int k = 0; k < 2; ++k) {
        const int bb = b + k;
        if (bb < 0 || bb >= V) continue;
        const float *row = sino + ((size_t)view * V + bb) * U;
        if (a >= 0 && a < U) t[2 * k] = row[a];
        if (a + 1 >= 0 && a + 1 < U) t[2 * k + 1] = row[a + 1];
    }
    S[idx] = make_float4(t[0], t[1] - t[0], t[2], t[3] - t[2]);
}

__global__ void k_relayout_sino3d_quad(const float *__restrict__ sino, int U, int V, int nangles,
                                       float4 *__restrict__ S) {
    relayout_sino3d_quad_at(sino, U, V, nangles, S, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Double-difference quads for the axial backprojector: element (b, a) holds
// s00, s01 - s00, s10 - s00 and (s11 - s10) - (s01 - s00) of the cells
// (row b, b + 1) x (column a, a + 1), zero outside the detector, so the
// bilinear value at fractions (wu, wv) is s00 + wu B + wv (C + wu D).
__device__ __forceinline__ void relayout_sino3d_qd_at(const float *__restrict__ sino, int U, int V,
                                                   int nangles, float4 *__restrict__ S,
                                                   long long idx) {
    const int PU = U + 2 * kP3, PV = V + 2 * kP3;
    if (idx >= (long long)PU * PV * nangles) return;
    const int a = (int)(idx % PU) - kP3;
    const long long r = idx / PU;
    const int b = (int)(r % PV) - kP3;
    const int view = (int)(r / PV);
    float t[4] = {0.f, 0.f, 0.f, 0.f};  // s00, s01, s10, s11
    for (int k = 0; k < 2; ++k) {
        const int bb = b + k;
        if (bb < 0 || bb >= V) continue;
        const float *row = sino + ((size_t)view * V + bb) * U;
        if (a >= 0 && a < U) t[2 * k] = row[a];
        if (a + 1 >= 0 && a + 1 < U) t[2 * k + 1] = row[a + 1];
    }
    S[idx] = make_float4(t[0], t[1] - t[0], t[2] - t[0], (t[3] - t[2]) - (t[1] - t[0]));
}

__global__ void k_relayout_sino3d_qd(const float *__restrict__ sino, int U, int V, int nangles,
                                     float4 *__restrict__ S) {
    relayout_sino3d_qd_at(sino, U, V, nangles, S, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------------------------ forward

// One thread per ray (u, v, view), the reference's ray set-up and float
// t-loop (forward_3d.hpp:56-93, intersection.h:12-28): the sample points are
// the reference's exactly up to FMA contraction; trilinear filtering is FP32
// in registers.  Rays that miss the box [-1, N+1]^3 write nothing.
__global__ void __launch_bounds__(256)
    k_fwd3d(const float2 *__restrict__ A, const float2 *__restrict__ B, float *__restrict__ sino,
            const float4 *__restrict__ torg, const float4 *__restrict__ tdu,
            const float4 *__restrict__ tdv, const float4 *__restrict__ tsrc, int X, int Y, int Z,
            int U, int V, bool exact_t) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.y * blockDim.y + threadIdx.y;
    const int view = blockIdx.z;
    if (iu >= U || iv >= V) return;
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
    // A non-finite ray (degenerate geometry) writes nothing rather than
    // walking an unbounded loop.
    if (!(h > 0.f) || !isfinite(tmax) || nsteps > (1 << 22)) return;

    // Choose the copy whose contiguous axis the warp's cells spread over.
    const bool xmajor = fabsf(dx) > fabsf(dz);
    const float sa = xmajor ? s.z : s.x, da = xmajor ? dz : dx;
    const float sc = xmajor ? s.x : s.z, dc = xmajor ? dx : dz;
    const float2 *L = xmajor ? B : A;
    const int Na = xmajor ? Z : X, Nc = xmajor ? X : Z;
    const int pa = Na + 2 * kP3, pb = Y + 2 * kP3;
    const unsigned acap = (unsigned)(Na + kP3), bcap = (unsigned)(Y + kP3),
                   ccap = (unsigned)(Nc + kP3);

    float acc = 0.f;
    float t = tmin;
    for (int k = 0; k <= nsteps + 1; ++k) {
        if (!(t <= tmax)) break;
        const float pa_ = fmaf(da, t, sa), pb_ = fmaf(dy, t, s.y), pc_ = fmaf(dc, t, sc);
        // texture coordinate p + 0.5 filtered at (p + 0.5) - 0.5 = p; indices
        // past the padded box clamp onto its zero border
        const FloorSplit fa = floor_split(pa_, -kP3), fb = floor_split(pb_, -kP3),
                         fc = floor_split(pc_, -kP3);
        const float wa = fa.frac, wb = fb.frac, wc = fc.frac;
        const float2 *p00 = L + ((size_t)min(fc.idx, ccap) * pb + min(fb.idx, bcap)) * pa +
                            min(fa.idx, acap);
        const float2 t00 = __ldg(p00);
        const float2 t10 = __ldg(p00 + pa);
        const float2 t01 = __ldg(p00 + (size_t)pa * pb);
        const float2 t11 = __ldg(p00 + (size_t)pa * pb + pa);
        const float l00 = fmaf(wa, t00.y, t00.x);
        const float l10 = fmaf(wa, t10.y, t10.x);
        const float l01 = fmaf(wa, t01.y, t01.x);
        const float l11 = fmaf(wa, t11.y, t11.x);
        const float m0 = fmaf(wb, l10 - l00, l00);
        const float m1 = fmaf(wb, l11 - l01, l01);
        acc += fmaf(wc, m1 - m0, m0);
        t = march_next(t, k, tmin, h, exact_t);
    }
    sino[((size_t)view * V + iv) * U + iu] = acc;
}

// ------------------------------------------------------------ forward, quads

// Ray set-up of forward_3d.hpp:56-81 (intersection.h:12-28) in the
// reference's FP32 operations.
struct Ray3 {
    float sx, sy, sz, dx, dy, dz, tmin, tmax, h;
    int nsteps;
    bool hit;
};

__device__ __forceinline__ Ray3 setup_ray3(const float4 o, const float4 du, const float4 dv,
                                           const float4 s, int iu, int iv, int X, int Y, int Z) {
    Ray3 r;
    const float fu = (float)iu, fv = (float)iv;
    const float detx = o.x + fu * du.x + fv * dv.x;
    const float dety = o.y + fu * du.y + fv * dv.y;
    const float detz = o.z + fu * du.z + fv * dv.z;
    r.sx = s.x, r.sy = s.y, r.sz = s.z;
    r.dx = detx - s.x, r.dy = dety - s.y, r.dz = detz - s.z;
    const float len = sqrtf(r.dx * r.dx + r.dy * r.dy + r.dz * r.dz);
    const long long nsamples = (long long)ceilf(__fdividef(len, 1.0f));
    float tmin = FLT_MIN, tmax = FLT_MAX;
    {
        const float t1 = __fdividef(-1.f - s.x, r.dx), t2 = __fdividef((float)(X + 1) - s.x, r.dx);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.y, r.dy), t2 = __fdividef((float)(Y + 1) - s.y, r.dy);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.z, r.dz), t2 = __fdividef((float)(Z + 1) - s.z, r.dz);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    r.tmin = tmin, r.tmax = tmax;
    r.hit = tmin <= tmax;
    r.nsteps = r.hit ? (int)ceilf((tmax - tmin) * (float)nsamples) : 0;
    r.h = r.hit ? (tmax - tmin) / (float)r.nsteps : 0.f;
    if (!(r.h > 0.f) || !isfinite(tmax) || r.nsteps > (1 << 22)) r.hit = false;
    return r;
}

// FP32 forward from the quad copies.  The reference's ray set-up and float
// t-loop (forward_3d.hpp:56-93), each sample trilinear in FP32: the floors
// by FP32 adds rounded toward -inf (bits of p + 1.5 * 2^23 = floor(p) +
// const), one offset for the three axes, two 16-byte loads (slices c and
// c + 1) and eight FMAs.  Rays that travel mostly along x read QB (columns
// z, slices x), the others QA, so that the warp's rays -- an 8 x 4 patch of
// detector cells -- spread along the contiguous axis.  Blocks are 32 x 8
// cells of one view, ordered cells fastest, then views, then bands of 8
// detector rows: the blocks resident at one time cover one band of rows of
// many views, whose rays cross a slab of the volume's y range that stays in
// L2.  The offset is clamped into the array (a guard; samples inside the box
// need no clamp).  With tex_warps > 0 (algorithm 5) the first tex_warps
// warps of each block take their rays through the texture unit instead
// (the reference's tex3D sampling): the texture path and the L1 load path
// then work side by side (3 of 8 warps: -8 % at 256^3, -21 % at 512^3
// against quads alone).
// UNR = 2 (default): two samples per iteration, both samples' loads (or
// texture fetches) issued before either is accumulated, so each warp keeps
// twice the memory requests in flight; the samples, their order of
// summation and the march's parameter sequence are those of UNR = 1, so the
// results are the same bits (the second sample's loads happen even when it
// lies past tmax, at an offset clamped into the array, and are then
// dropped).  -2 % at 256^3, -0.7 % at 512^3 (the texture warps gain; the
// quads alone do not change; four fetches per iteration: no better).
// Block `lin` of the launch order above (the batched forward passes each
// problem's own block index).
template <int UNR>
__device__ __forceinline__ void fwd3d_quad_block(
    const float4 *__restrict__ QA, const float4 *__restrict__ QB, float *__restrict__ sino,
    const float4 *__restrict__ torg, const float4 *__restrict__ tdu,
    const float4 *__restrict__ tdv, const float4 *__restrict__ tsrc, int X, int Y, int Z, int U,
    int V, int P, int utiles, cudaTextureObject_t tex, int tex_warps, bool exact_t, int lin) {
    const int ut = lin % utiles, rest = lin / utiles;
    const int view = rest % P, band = rest / P;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int iu = ut * 32 + (warp & 3) * 8 + (lane & 7);
    const int iv = band * 8 + (warp >> 2) * 4 + (lane >> 3);
    if (iu >= U || iv >= V) return;
    const Ray3 r = setup_ray3(torg[view], tdu[view], tdv[view], tsrc[view], iu, iv, X, Y, Z);
    if (!r.hit) return;
    if (warp < tex_warps) {
        // this warp's rays through the texture unit (trilinear, 8-bit weights)
        // UNR fetches per iteration (their sample parameters in sequence),
        // accumulated in order up to the first one past tmax
        float acc = 0.f, t = r.tmin;
        const int kend = r.nsteps + 2;
        for (int k = 0; k < kend; k += UNR) {
            if (!(t <= r.tmax)) break;
            float ts[UNR], sv[UNR];
            ts[0] = t;
#pragma unroll
            for (int j = 1; j < UNR; ++j) ts[j] = march_next(ts[j - 1], k + j - 1, r.tmin, r.h, exact_t);
#pragma unroll
            for (int j = 0; j < UNR; ++j)
                sv[j] = tex3D<float>(tex, fmaf(r.dx, ts[j], r.sx) + 0.5f,
                                     fmaf(r.dy, ts[j], r.sy) + 0.5f,
                                     fmaf(r.dz, ts[j], r.sz) + 0.5f);
            acc += sv[0];
            bool more = true;
#pragma unroll
            for (int j = 1; j < UNR; ++j) {
                more = more && k + j < kend && ts[j] <= r.tmax;
                if (more) acc += sv[j];
            }
            if (!more) break;
            t = march_next(ts[UNR - 1], k + UNR - 1, r.tmin, r.h, exact_t);
        }
        sino[((size_t)view * V + iv) * U + iu] = acc;
        return;
    }
    const bool xmajor = fabsf(r.dx) > fabsf(r.dz);
    const float4 *Q = xmajor ? QB : QA;
    const float sa = xmajor ? r.sz : r.sx, da = xmajor ? r.dz : r.dx;
    const float sc = xmajor ? r.sx : r.sz, dc = xmajor ? r.dx : r.dz;
    const unsigned PA = (unsigned)((xmajor ? Z : X) + kQP), PB = (unsigned)(Y + kQP);
    const unsigned PC = (unsigned)((xmajor ? X : Z) + kQP);
    const unsigned slice = PA * PB;
    const unsigned maxoff = (PC - 1) * slice - 1;  // off + slice stays inside
    constexpr float kMagic = 12582912.0f;          // 1.5 * 2^23
    const unsigned base = 0x4B400000u - (unsigned)kP3;
    // off = (bits_c - base) slice + (bits_b - base) PA + (bits_a - base), mod 2^32
    const unsigned K = base * slice + base * PA + base;
    const float4 *Q1 = Q + slice;
    // one sample at parameter t: its two quads' loads, then its value
    struct Fetch {
        float4 q0, q1;
        float wa, wb, wc;
    };
    auto fetch = [&](float t) {
        Fetch f;
        const float pa = fmaf(da, t, sa), pb = fmaf(r.dy, t, r.sy), pc = fmaf(dc, t, sc);
        const float ta = __fadd_rd(pa, kMagic), tb = __fadd_rd(pb, kMagic),
                    tc = __fadd_rd(pc, kMagic);
        f.wa = __fadd_rn(pa, -__fadd_rn(ta, -kMagic));
        f.wb = __fadd_rn(pb, -__fadd_rn(tb, -kMagic));
        f.wc = __fadd_rn(pc, -__fadd_rn(tc, -kMagic));
        unsigned off = __float_as_uint(tc) * slice + __float_as_uint(tb) * PA +
                       (__float_as_uint(ta) - K);
        off = min(off, maxoff);
        f.q0 = __ldg(Q + off), f.q1 = __ldg(Q1 + off);
        return f;
    };
    auto value = [](const Fetch &f) {
        const float l0 = fmaf(f.wa, f.q0.y, f.q0.x), g0 = fmaf(f.wa, f.q0.w, f.q0.z);
        const float l1 = fmaf(f.wa, f.q1.y, f.q1.x), g1 = fmaf(f.wa, f.q1.w, f.q1.z);
        const float m0 = fmaf(f.wb, g0, l0), m1 = fmaf(f.wb, g1, l1);
        return fmaf(f.wc, m1 - m0, m0);
    };
    // the quads: two samples per iteration whenever UNR >= 2
    constexpr int QU = UNR >= 2 ? 2 : 1;
    float acc = 0.f, t = r.tmin;
    const int kend = r.nsteps + 2;
    for (int k = 0; k < kend; k += QU) {
        if (!(t <= r.tmax)) break;
        const Fetch f0 = fetch(t);
        if constexpr (QU == 2) {
            const float t1 = march_next(t, k, r.tmin, r.h, exact_t);
            const Fetch f1 = fetch(t1);
            acc += value(f0);
            if (!(k + 1 < kend && t1 <= r.tmax)) break;
            acc += value(f1);
            t = march_next(t1, k + 1, r.tmin, r.h, exact_t);
        } else {
            acc += value(f0);
            t = march_next(t, k, r.tmin, r.h, exact_t);
        }
    }
    sino[((size_t)view * V + iv) * U + iu] = acc;
}

template <int UNR>
__global__ void __launch_bounds__(256)
    k_fwd3d_quad(const float4 *__restrict__ QA, const float4 *__restrict__ QB,
                 float *__restrict__ sino, const float4 *__restrict__ torg,
                 const float4 *__restrict__ tdu, const float4 *__restrict__ tdv,
                 const float4 *__restrict__ tsrc, int X, int Y, int Z, int U, int V, int P,
                 int utiles, cudaTextureObject_t tex, int tex_warps, bool exact_t) {
    fwd3d_quad_block<UNR>(QA, QB, sino, torg, tdu, tdv, tsrc, X, Y, Z, U, V, P, utiles, tex,
                          tex_warps, exact_t, blockIdx.x);
}

// ------------------------------------------------------------ backward

constexpr int kBZ = 8;         // voxels per thread along z
constexpr int kBViews = 64;    // view tables staged per pass

struct BwdTab {
    float4 o, dx, dy, dz;
};

// Block = 32 (x) x 8 (y) threads, each with a run of kBZ voxels along z
// (PK: taken two at a time with packed FP32 instructions, 11 % faster at
// 512^3 than one at a time; MAGIC: the detector floor by FP32 adds,
// floor_split two at a time, another 4 %).
// Blocks are visited brick by brick (2 x 8 x 8 tiles) so that the blocks
// resident at one time cover a compact region of the volume and share the
// detector footprint they read from L2.  Per voxel and view: the reference's
// ray/plane intersection (backward_3d.hpp:78-94) -- the ray direction is
// stepped along z from the run's first voxel -- then a bilinear sample of the
// difference-encoded pair-packed projection in two 8-byte loads and three
// FMAs, accumulated in registers; the volume is read and written once.
template <bool PK, bool MAGIC, bool QS>
__device__ __forceinline__ void bwd3d_block(
    float *__restrict__ vol, const void *__restrict__ Sv, const float4 *__restrict__ torg,
    const float4 *__restrict__ tdx, const float4 *__restrict__ tdy,
    const float4 *__restrict__ tdz, float srcx, float srcy, float srcz, float zplane, float hu,
    float hv, int X, int Y, int Z, int U, int V, int nangles, int tiles_x, int tiles_y,
    int tiles_z, int lin) {
    __shared__ BwdTab stab[kBViews];
    const float2 *S = static_cast<const float2 *>(Sv);
    const float4 *SQ = static_cast<const float4 *>(Sv);  // QS: row-pair quads
    // brick-ordered tile index
    constexpr int BX = 2, BY = 8, BZ = 8;
    const int bricks_x = (tiles_x + BX - 1) / BX, bricks_y = (tiles_y + BY - 1) / BY;
    const int brick = lin / (BX * BY * BZ), in = lin % (BX * BY * BZ);
    const int bx = brick % bricks_x, by = (brick / bricks_x) % bricks_y,
              bz = brick / (bricks_x * bricks_y);
    const int tx_ = bx * BX + in % BX, ty_ = by * BY + (in / BX) % BY, tz_ = bz * BZ + in / (BX * BY);
    const bool tile_ok = tx_ < tiles_x && ty_ < tiles_y && tz_ < tiles_z;

    const int x = tx_ * 32 + threadIdx.x, y = ty_ * 8 + threadIdx.y, z0 = tz_ * kBZ;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const float fx = (float)x, fy = (float)y, fz0 = (float)z0;
    const int PU = U + 2 * kP3, PV = V + 2 * kP3;
    const unsigned ucap = (unsigned)(U + kP3), vcap = (unsigned)(V + kP3);
    const float num = zplane - srcz;
    // detector coordinate minus the texel-centre half: (dir t + s) + U/2 - 1/2
    const float su = srcx + hu - 0.5f, sv = srcy + hv - 0.5f;

    float acc[kBZ];
#pragma unroll
    for (int k = 0; k < kBZ; ++k) acc[k] = 0.f;

    for (int v0 = 0; v0 < nangles; v0 += kBViews) {
        const int nv = min(kBViews, nangles - v0);
        __syncthreads();
        for (int i = tid; i < nv * 4; i += 256) {
            const int j = i >> 2, f = i & 3;
            const float4 *src = f == 0 ? torg : f == 1 ? tdx : f == 2 ? tdy : tdz;
            reinterpret_cast<float4 *>(&stab[j])[f] = src[v0 + j];
        }
        __syncthreads();
        if (!tile_ok) continue;
        for (int j = 0; j < nv; ++j) {
            const BwdTab tb = stab[j];
            // direction source -> voxel (x, y, z0), P = o + x dx + y dy + z dz
            float dirx = fmaf(fz0, tb.dz.x, fmaf(fy, tb.dy.x, fmaf(fx, tb.dx.x, tb.o.x))) - srcx;
            float diry = fmaf(fz0, tb.dz.y, fmaf(fy, tb.dy.y, fmaf(fx, tb.dx.y, tb.o.y))) - srcy;
            float dirz = fmaf(fz0, tb.dz.z, fmaf(fy, tb.dy.z, fmaf(fx, tb.dx.z, tb.o.z))) - srcz;
            const float2 *plane = S + (size_t)(v0 + j) * PU * PV;
            const float4 *planeQ = SQ + (size_t)(v0 + j) * PU * PV;
            if constexpr (PK) {
                // two voxels (k, k + 1) per packed FP32 instruction
                const float2 step_x = make_float2(2.f * tb.dz.x, 2.f * tb.dz.x);
                const float2 step_y = make_float2(2.f * tb.dz.y, 2.f * tb.dz.y);
                const float2 step_z = make_float2(2.f * tb.dz.z, 2.f * tb.dz.z);
                float2 DX = make_float2(dirx, dirx + tb.dz.x);
                float2 DY = make_float2(diry, diry + tb.dz.y);
                float2 DZ = make_float2(dirz, dirz + tb.dz.z);
                const float2 N2 = make_float2(num, num), SU = make_float2(su, su),
                             SV = make_float2(sv, sv);
#pragma unroll
                for (int k = 0; k < kBZ; k += 2) {
                    const float2 t = __fmul2_rn(
                        N2, make_float2(rcp_approx(DZ.x), rcp_approx(DZ.y)));
                    const float2 ub = __ffma2_rn(DX, t, SU), vb = __ffma2_rn(DY, t, SV);
                    float2 wu, wv;
                    unsigned cu0, cu1, cv0, cv1;
                    if constexpr (MAGIC) {
                        // floor by packed FP32 adds (floor_split, two at a time)
                        const float2 m = make_float2(12582912.0f, 12582912.0f);
                        const float2 h = make_float2(-0.5f, -0.5f), nm = make_float2(-12582912.0f,
                                                                                     -12582912.0f);
                        const float2 tu = __fadd2_rn(__fadd2_rn(ub, h), m);
                        const float2 tv = __fadd2_rn(__fadd2_rn(vb, h), m);
                        const float2 ku = __fadd2_rn(tu, nm), kv = __fadd2_rn(tv, nm);
                        wu = __fadd2_rn(ub, make_float2(-ku.x, -ku.y));
                        wv = __fadd2_rn(vb, make_float2(-kv.x, -kv.y));
                        const unsigned base = 0x4B400000u - (unsigned)kP3;
                        cu0 = min(__float_as_uint(tu.x) - base, ucap);
                        cu1 = min(__float_as_uint(tu.y) - base, ucap);
                        cv0 = min(__float_as_uint(tv.x) - base, vcap);
                        cv1 = min(__float_as_uint(tv.y) - base, vcap);
                    } else {
                        const int iu0 = __float2int_rd(ub.x), iu1 = __float2int_rd(ub.y);
                        const int iv0 = __float2int_rd(vb.x), iv1 = __float2int_rd(vb.y);
                        wu = __fadd2_rn(ub, make_float2(-(float)iu0, -(float)iu1));
                        wv = __fadd2_rn(vb, make_float2(-(float)iv0, -(float)iv1));
                        cu0 = min((unsigned)(iu0 + kP3), ucap), cu1 = min((unsigned)(iu1 + kP3), ucap);
                        cv0 = min((unsigned)(iv0 + kP3), vcap), cv1 = min((unsigned)(iv1 + kP3), vcap);
                    }
                    float2 a0, b0, a1, b1;
                    if constexpr (QS) {
                        const float4 w0 = __ldg(planeQ + cv0 * PU + cu0);
                        const float4 w1 = __ldg(planeQ + cv1 * PU + cu1);
                        a0 = make_float2(w0.x, w0.y), b0 = make_float2(w0.z, w0.w);
                        a1 = make_float2(w1.x, w1.y), b1 = make_float2(w1.z, w1.w);
                    } else {
                        const float2 *q0 = plane + cv0 * PU + cu0;
                        const float2 *q1 = plane + cv1 * PU + cu1;
                        a0 = __ldg(q0), b0 = __ldg(q0 + PU);
                        a1 = __ldg(q1), b1 = __ldg(q1 + PU);
                    }
                    const float2 l0 = make_float2(fmaf(wu.x, a0.y, a0.x), fmaf(wu.y, a1.y, a1.x));
                    const float2 l1 = make_float2(fmaf(wu.x, b0.y, b0.x), fmaf(wu.y, b1.y, b1.x));
                    const float2 m =
                        __ffma2_rn(wv, __fadd2_rn(l1, make_float2(-l0.x, -l0.y)), l0);
                    const float2 s2 = __fadd2_rn(make_float2(acc[k], acc[k + 1]), m);
                    acc[k] = s2.x, acc[k + 1] = s2.y;
                    DX = __fadd2_rn(DX, step_x);
                    DY = __fadd2_rn(DY, step_y);
                    DZ = __fadd2_rn(DZ, step_z);
                }
            } else {
#pragma unroll
                for (int k = 0; k < kBZ; ++k) {
                    const float t = num * rcp_approx(dirz);
                    const float ub = fmaf(dirx, t, su), vb = fmaf(diry, t, sv);
                    const int iu = __float2int_rd(ub), iv = __float2int_rd(vb);
                    const float wu = ub - (float)iu, wv = vb - (float)iv;
                    const unsigned cu = min((unsigned)(iu + kP3), ucap);
                    const unsigned cv = min((unsigned)(iv + kP3), vcap);
                    const float2 *q = plane + cv * PU + cu;
                    const float2 a = __ldg(q), b = __ldg(q + PU);
                    const float l0 = fmaf(wu, a.y, a.x);
                    const float l1 = fmaf(wu, b.y, b.x);
                    acc[k] += fmaf(wv, l1 - l0, l0);
                    dirx += tb.dz.x;
                    diry += tb.dz.y;
                    dirz += tb.dz.z;
                }
            }
        }
    }
    if (!tile_ok || x >= X || y >= Y) return;
#pragma unroll
    for (int k = 0; k < kBZ; ++k) {
        const int z = z0 + k;
        if (z < Z) vol[((size_t)z * Y + y) * X + x] += acc[k];
    }
}

template <bool PK, bool MAGIC = false, bool QS = false>
__global__ void __launch_bounds__(256)
    k_bwd3d(float *__restrict__ vol, const void *__restrict__ Sv,
            const float4 *__restrict__ torg, const float4 *__restrict__ tdx,
            const float4 *__restrict__ tdy, const float4 *__restrict__ tdz, float srcx,
            float srcy, float srcz, float zplane, float hu, float hv, int X, int Y, int Z, int U,
            int V, int nangles, int tiles_x, int tiles_y, int tiles_z) {
    bwd3d_block<PK, MAGIC, QS>(vol, Sv, torg, tdx, tdy, tdz, srcx, srcy, srcz, zplane, hu, hv, X,
                               Y, Z, U, V, nangles, tiles_x, tiles_y, tiles_z, blockIdx.x);
}

// Views per launch of k_bwd3d_ax: their tables travel as a 30 KB kernel
// parameter (the limit is 32 KB).
constexpr int kAxViews = 768;
struct AxViewParams {
    float4 p0[kAxViews];  // source -> voxel (0, 0, 0): x, y, z; v component of the y step
    float4 p1[kAxViews];  // x step; z step's x
    float2 p2[kAxViews];  // z step's y, z
};

// Backprojection for geometries whose every view maps the volume's y axis
// onto the detector's v axis (the y step of the view table is (0, dy, 0)):
// circular orbits about y without detector tilt.  Along a run of voxels in
// y the ray's detector-normal and u components are then constant, so a
// thread takes RUN voxels along y with one reciprocal, one u floor and one
// detector column per view, and per voxel only the v coordinate: the floor
// by an FP32 add rounded toward -inf (the magic 1.5 * 2^23 has unit
// spacing, so the sum's bits are floor(v) + const exactly), one 16-byte
// load of a double-difference quad and three FMAs.  Block = 256 threads
// over 32 (x) x 8 (z) voxels, each warp on an 8 x 4 patch so its lanes read
// a compact piece of the projection; blocks are visited in bricks of 2 x 8
// x 8 tiles like k_bwd3d.  The per-view tables are a kernel parameter, read
// through the constant cache uniformly across the warp: no shared-memory
// staging or barriers, and the table reads stay off the L1's register
// write-back path, which the projection loads saturate (-9 % against
// staging them in shared memory).  Same ray/plane intersection as the
// reference (backward_3d.hpp:78-94).
// Block `lin` of the brick order over views [0, nv): tab(j) gives view j's
// (p0, p1, p2), from the kernel parameter or (batched) from device memory.
template <int RUN, class Tab>
__device__ __forceinline__ void bwd3d_ax_block(float *__restrict__ vol,
                                               const float4 *__restrict__ SQ, const Tab &tab,
                                               int nv, float num, float su, float sv, int X,
                                               int Y, int Z, int U, int V, int tiles_x,
                                               int tiles_y, int tiles_z, int lin) {
    constexpr int BX = 2, BY = 8, BZ = 8;
    const int bricks_x = (tiles_x + BX - 1) / BX, bricks_y = (tiles_y + BY - 1) / BY;
    const int brick = lin / (BX * BY * BZ), in = lin % (BX * BY * BZ);
    const int bx = brick % bricks_x, by = (brick / bricks_x) % bricks_y,
              bz = brick / (bricks_x * bricks_y);
    const int tx_ = bx * BX + in % BX, ty_ = by * BY + (in / BX) % BY, tz_ = bz * BZ + in / (BX * BY);
    if (tx_ >= tiles_x || ty_ >= tiles_y || tz_ >= tiles_z) return;

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int x = tx_ * 32 + (warp & 3) * 8 + (lane & 7);
    const int z = tz_ * 8 + (warp >> 2) * 4 + (lane >> 3);
    const int y0 = ty_ * RUN;
    const float fx = (float)x, fz = (float)z, fy0 = (float)y0;
    const int PU = U + 2 * kP3, PV = V + 2 * kP3;
    const size_t plane_elems = (size_t)PU * PV;
    const unsigned rowb = (unsigned)PU * (unsigned)sizeof(float4);
    const unsigned ucap = (unsigned)(U + kP3), vcap = (unsigned)(V + kP3);
    const unsigned base = 0x4B400000u - (unsigned)kP3;  // bits of 1.5 * 2^23 - kP3
    constexpr float kMagic = 12582912.0f;              // 1.5 * 2^23
    const float2 M2 = make_float2(kMagic, kMagic), NEG1 = make_float2(-1.f, -1.f);

    float acc[RUN];
#pragma unroll
    for (int k = 0; k < RUN; ++k) acc[k] = 0.f;

    const float4 *plane = SQ;
    for (int j = 0; j < nv; ++j, plane += plane_elems) {
        float4 p0, p1;
        float2 p2;
        tab(j, p0, p1, p2);
        const float dirx = fmaf(fz, p1.w, fmaf(fx, p1.x, p0.x));
        const float diry = fmaf(fy0, p0.w, fmaf(fz, p2.x, fmaf(fx, p1.y, p0.y)));
        const float dirz = fmaf(fz, p2.y, fmaf(fx, p1.z, p0.z));
        const float t = __fdividef(num, dirz);
        const float ub = fmaf(dirx, t, su);
        const float vb0 = fmaf(diry, t, sv), dvb = p0.w * t;
        const float tu = __fadd_rd(ub, kMagic);
        const float wu = __fadd_rn(ub, -__fadd_rn(tu, -kMagic));
        const unsigned cu = min(__float_as_uint(tu) - base, ucap);
        const float4 *col = plane + cu;
        float2 vb = make_float2(vb0, vb0 + dvb);
        const float2 step = make_float2(2.f * dvb, 2.f * dvb);
#pragma unroll
        for (int k = 0; k < RUN; k += 2) {
            const float2 tv = __fadd2_rd(vb, M2);
            const float2 wv = __fadd2_rn(vb, __ffma2_rn(tv, NEG1, M2));  // vb - floor(vb)
            const unsigned c0 = min(__float_as_uint(tv.x) - base, vcap);
            const unsigned c1 = min(__float_as_uint(tv.y) - base, vcap);
            const float4 q0 = __ldg(reinterpret_cast<const float4 *>(
                reinterpret_cast<const char *>(col) + (size_t)c0 * rowb));
            const float4 q1 = __ldg(reinterpret_cast<const float4 *>(
                reinterpret_cast<const char *>(col) + (size_t)c1 * rowb));
            const float2 l0 = make_float2(fmaf(wu, q0.y, q0.x), fmaf(wu, q1.y, q1.x));
            const float2 g = make_float2(fmaf(wu, q0.w, q0.z), fmaf(wu, q1.w, q1.z));
            const float2 a = __ffma2_rn(wv, g, __fadd2_rn(make_float2(acc[k], acc[k + 1]), l0));
            acc[k] = a.x, acc[k + 1] = a.y;
            vb = __fadd2_rn(vb, step);
        }
    }
    if (x >= X || z >= Z) return;
#pragma unroll
    for (int k = 0; k < RUN; ++k) {
        const int y = y0 + k;
        if (y < Y) vol[((size_t)z * Y + y) * X + x] += acc[k];
    }
}

template <int RUN, int MINB>
__global__ void __launch_bounds__(256, MINB)
    k_bwd3d_ax(float *__restrict__ vol, const float4 *__restrict__ SQ,
                const __grid_constant__ AxViewParams tab, int nv, float num, float su, float sv,
                int X, int Y, int Z, int U, int V, int tiles_x, int tiles_y, int tiles_z) {
    const auto param_tab = [&](int j, float4 &p0, float4 &p1, float2 &p2) {
        p0 = tab.p0[j], p1 = tab.p1[j], p2 = tab.p2[j];
    };
    bwd3d_ax_block<RUN>(vol, SQ, param_tab, nv, num, su, sv, X, Y, Z, U, V, tiles_x, tiles_y,
                        tiles_z, blockIdx.x);
}

}  // namespace

// ------------------------------------------------------------ launchers

// cudaMalloc that reports an out-of-memory failure as false (clearing the
// error) and other failures as a thrown status through *rc.
static bool try_malloc_or_oom(void **ptr, size_t bytes, int *rc) {
    const cudaError_t e = cudaMalloc(ptr, bytes);
    if (e == cudaSuccess) return true;
    *ptr = nullptr;
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        return false;
    }
    *rc = set_error(CG_ERR_CUDA, cudaGetErrorString(e));
    return false;
}

int ensure_plan3d_scratch(Plan3d &p, bool fwd, bool bwd) {
    if (fwd && !p.d_volA) {
        const size_t n = (size_t)(p.X + 2 * kP3) * (p.Y + 2 * kP3) * (p.Z + 2 * kP3);
        CG_TRY_CUDA(cudaMalloc(&p.d_volA, n * sizeof(float2)));
        CG_TRY_CUDA(cudaMalloc(&p.d_volB, n * sizeof(float2)));
        p.volA_elems = p.volB_elems = n;
    }
    if (bwd) {
        // one of the two re-laid projections, as the plan's variant reads it
        const size_t n = (size_t)(p.U + 2 * kP3) * (p.V + 2 * kP3) * p.nangles;
        p.sinoP_elems = n;
        if (p.reads_quads() && !p.d_sinoQ) {
            int rc = CG_OK;
            if (!try_malloc_or_oom((void **)&p.d_sinoQ, n * sizeof(float4), &rc)) {
                if (rc) return rc;
                // no room for the 16-byte quads: the general kernel on 8-byte
                // pairs (half the memory) from now on
                p.algo_bwd = 0, p.bwd_packed = 2;
            }
        }
        if (!p.reads_quads() && !p.d_sinoP)
            CG_TRY_CUDA(cudaMalloc(&p.d_sinoP, n * sizeof(float2)));
    }
    return CG_OK;
}

int launch_forward3d(const Plan3d &p, const float *vol, float *sino, cudaStream_t s) {
    {
        const long long n = (long long)p.volA_elems;
        k_relayout3d_A<<<ceil_div(n, 256), 256, 0, s>>>(vol, p.X, p.Y, p.Z, p.d_volA);
        CG_TRY_CUDA(cudaGetLastError());
        dim3 g(ceil_div(p.X + 2 * kP3, 32), ceil_div(p.Z + 2 * kP3, 32), p.Y + 2 * kP3);
        k_relayout3d_B<<<g, dim3(32, 8), 0, s>>>(vol, p.X, p.Y, p.Z, p.d_volB);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (p.nangles > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    dim3 grid(ceil_div(p.U, 32), ceil_div(p.V, 8), p.nangles);
    k_fwd3d<<<grid, dim3(32, 8), 0, s>>>(p.d_volA, p.d_volB, sino, p.d_forg, p.d_fdu, p.d_fdv,
                                         p.d_fsrc, p.X, p.Y, p.Z, p.U, p.V, p.exact_t);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_forward3d_quad(Plan3d &p, const float *vol, float *sino, cudaStream_t s) {
    const size_t n = (size_t)(p.X + kQP) * (p.Y + kQP) * (p.Z + kQP);
    // the kernel's offsets are 32-bit: larger volumes take the texture unit
    if (n >= (1ull << 32)) return launch_forward3d_tex(p, vol, sino, s);
    if (!p.d_volQA) {
        int rc = CG_OK;
        if (!try_malloc_or_oom((void **)&p.d_volQA, n * sizeof(float4), &rc) ||
            !try_malloc_or_oom((void **)&p.d_volQB, n * sizeof(float4), &rc)) {
            if (p.d_volQA) cudaFree(p.d_volQA);
            p.d_volQA = nullptr;
            if (rc) return rc;
            // no room for the two quad copies: algorithm 4 continues as the
            // register forward (the same samples and weights, 8-byte pair
            // copies), algorithm 5 as the texture forward
            if (p.algo_fwd == 4) {
                p.algo_fwd = 0;
                if ((rc = ensure_plan3d_scratch(p, true, false))) return rc;
                return launch_forward3d(p, vol, sino, s);
            }
            p.algo_fwd = 1;
            return launch_forward3d_tex(p, vol, sino, s);
        }
    }
    k_relayout3d_qa<<<ceil_div((long long)n, 256), 256, 0, s>>>(vol, p.X, p.Y, p.Z, p.d_volQA);
    CG_TRY_CUDA(cudaGetLastError());
    dim3 g(ceil_div(p.Z + kQP, 32), ceil_div(p.X + kQP, 32), p.Y + kQP);
    k_relayout3d_qb<<<g, dim3(32, 8), 0, s>>>(vol, p.X, p.Y, p.Z, p.d_volQB);
    CG_TRY_CUDA(cudaGetLastError());
    const int utiles = ceil_div(p.U, 32);
    const long long blocks = (long long)utiles * p.nangles * ceil_div(p.V, 8);
    if (blocks >= (1ll << 31)) return set_error(CG_ERR_INVALID, "too many rays for one launch");
    // algorithm 5: some warps of each block sample through the texture unit
    const int tex_warps = p.algo_fwd == 5 ? p.fwd_tex_warps : 0;
    cudaTextureObject_t tex = 0;
    if (tex_warps > 0) {
        int rc = upload_volume_texture3(p, vol, s);
        if (rc) return rc;
        tex = p.tex3;
    }
    auto kernel = p.fwd_unroll == 2 ? k_fwd3d_quad<2> : k_fwd3d_quad<1>;
    kernel<<<(unsigned)blocks, 256, 0, s>>>(p.d_volQA, p.d_volQB, sino, p.d_forg, p.d_fdu,
                                            p.d_fdv, p.d_fsrc, p.X, p.Y, p.Z, p.U, p.V,
                                            p.nangles, utiles, tex, tex_warps, p.exact_t);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_backward3d(const Plan3d &p, float *vol, const float *sino, cudaStream_t s) {
    const float zplane = p.DSO - p.DSD;
    const float hu = (float)(p.U / 2), hv = (float)(p.V / 2);
    if (p.runs_axial()) {
        const long long n = (long long)p.sinoP_elems;
        k_relayout_sino3d_qd<<<ceil_div(n, 256), 256, 0, s>>>(sino, p.U, p.V, p.nangles,
                                                              p.d_sinoQ);
        CG_TRY_CUDA(cudaGetLastError());
        constexpr int run = 8;
        const int tiles_x = ceil_div(p.X, 32), tiles_y = ceil_div(p.Y, run),
                  tiles_z = ceil_div(p.Z, 8);
        const int bricks = ceil_div(tiles_x, 2) * ceil_div(tiles_y, 8) * ceil_div(tiles_z, 8);
        const size_t plane = (size_t)(p.U + 2 * kP3) * (p.V + 2 * kP3);
        // runs of 8 voxels at <= 48 registers (5 blocks per SM)
        auto kernel = k_bwd3d_ax<run, 5>;
        // the view tables travel as a kernel parameter, kAxViews per launch
        AxViewParams tab{};
        for (int c0 = 0; c0 < p.nangles; c0 += kAxViews) {
            const int nv = std::min(kAxViews, p.nangles - c0);
            for (int j = 0; j < nv; ++j) {
                const float *a = p.ax_views.data() + (size_t)(c0 + j) * 10;
                tab.p0[j] = make_float4(a[0], a[1], a[2], a[9]);
                tab.p1[j] = make_float4(a[3], a[4], a[5], a[6]);
                tab.p2[j] = make_float2(a[7], a[8]);
            }
            kernel<<<bricks * 128, 256, 0, s>>>(vol, p.d_sinoQ + plane * c0, tab, nv,
                                                zplane - p.bsrc[2], p.bsrc[0] + hu - 0.5f,
                                                p.bsrc[1] + hv - 0.5f, p.X, p.Y, p.Z, p.U, p.V,
                                                tiles_x, tiles_y, tiles_z);
            CG_TRY_CUDA(cudaGetLastError());
        }
        return CG_OK;
    }
    const bool quad = p.bwd_packed == 3;
    {
        const long long n = (long long)p.sinoP_elems;
        if (quad) {
            k_relayout_sino3d_quad<<<ceil_div(n, 256), 256, 0, s>>>(sino, p.U, p.V, p.nangles,
                                                                    p.d_sinoQ);
        } else {
            k_relayout_sino3d<<<ceil_div(n, 256), 256, 0, s>>>(sino, p.U, p.V, p.nangles,
                                                               p.d_sinoP);
        }
        CG_TRY_CUDA(cudaGetLastError());
    }
    const int tiles_x = ceil_div(p.X, 32), tiles_y = ceil_div(p.Y, 8), tiles_z = ceil_div(p.Z, kBZ);
    const int bricks = ceil_div(tiles_x, 2) * ceil_div(tiles_y, 8) * ceil_div(tiles_z, 8);
    // row-pair quads (default), or 8-byte pairs where the quads did not fit
    auto kernel = quad ? k_bwd3d<true, true, true> : k_bwd3d<true, true>;
    kernel<<<bricks * 128, dim3(32, 8), 0, s>>>(
        vol, quad ? (const void *)p.d_sinoQ : (const void *)p.d_sinoP, p.d_borg, p.d_bdx,
        p.d_bdy, p.d_bdz, p.bsrc[0], p.bsrc[1], p.bsrc[2], zplane, hu, hv, p.X, p.Y, p.Z, p.U, p.V, p.nangles, tiles_x, tiles_y, tiles_z);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

// ------------------------------------------------------------ batches

// Many 3D problems per launch: stage s of problem i owns the blocks
// [start[i], start[i + 1]) of the stage's launch; each block finds its
// problem by binary search over the starts and runs the single-problem
// block code on that problem's buffers with its own block index, so the
// results are those of the single-problem kernels bit for bit.
namespace {

__global__ void __launch_bounds__(256)
    k_batch3d_qa(const Prob3d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    relayout3d_qa_at(q.vol, q.X, q.Y, q.Z, q.QA,
                     (long long)(blockIdx.x - start[i]) * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(256)
    k_batch3d_qb(const Prob3d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    const int lin = blockIdx.x - start[i];
    const int ga = (q.Z + kQP + 31) / 32, gc = (q.X + kQP + 31) / 32;
    relayout3d_qb_tile(q.vol, q.X, q.Y, q.Z, q.QB, lin % ga, (lin / ga) % gc, lin / (ga * gc));
}

__global__ void __launch_bounds__(256, 6)
    k_batch3d_fwd(const Prob3d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    fwd3d_quad_block<2>(q.QA, q.QB, q.sino, q.forg, q.fdu, q.fdv, q.fsrc, q.X, q.Y, q.Z, q.U,
                        q.V, q.P, q.utiles, q.tex, q.tex_warps, q.exact_t != 0,
                        blockIdx.x - start[i]);
}

__global__ void __launch_bounds__(256)
    k_batch3d_relayout_sino(const Prob3d *__restrict__ probs, const int *__restrict__ start,
                            int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    const long long idx = (long long)(blockIdx.x - start[i]) * blockDim.x + threadIdx.x;
    if (q.axial)
        relayout_sino3d_qd_at(q.sino, q.U, q.V, q.P, q.sinoQ, idx);
    else
        relayout_sino3d_quad_at(q.sino, q.U, q.V, q.P, q.sinoQ, idx);
}

// The axial backprojection over every view of the problem, kAxViews views
// at a time with the running sum added into the volume after each (as the
// single-problem launches do), the view tables read from device memory.
template <int RUN>
__global__ void __launch_bounds__(256, 5)
    k_batch3d_bwd_ax(const Prob3d *__restrict__ probs, const int *__restrict__ start,
                     int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    const int lin = blockIdx.x - start[i];
    const size_t plane = (size_t)(q.U + 2 * kP3) * (q.V + 2 * kP3);
    for (int c0 = 0; c0 < q.P; c0 += kAxViews) {
        const int nv = min(kAxViews, q.P - c0);
        const float4 *a0 = q.ax0 + c0, *a1 = q.ax1 + c0;
        const float2 *a2 = q.ax2 + c0;
        const auto tab = [&](int j, float4 &p0, float4 &p1, float2 &p2) {
            p0 = __ldg(a0 + j), p1 = __ldg(a1 + j), p2 = __ldg(a2 + j);
        };
        bwd3d_ax_block<RUN>(q.vol, q.sinoQ + plane * c0, tab, nv, q.num, q.su, q.sv, q.X, q.Y,
                            q.Z, q.U, q.V, q.tiles_x, q.tiles_y, q.tiles_z, lin);
    }
}

__global__ void __launch_bounds__(256, 5)
    k_batch3d_bwd(const Prob3d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob3d &q = probs[i];
    bwd3d_block<true, true, true>(q.vol, q.sinoQ, q.borg, q.bdx, q.bdy, q.bdz, q.bsx, q.bsy,
                                  q.bsz, q.zplane, q.hu, q.hv, q.X, q.Y, q.Z, q.U, q.V, q.P,
                                  q.tiles_x, q.tiles_y, q.tiles_z, blockIdx.x - start[i]);
}

}  // namespace

int bind_batch3d_problem(Plan3d &p, float *vol, float *sino, float *ax, Prob3d *q,
                         int blocks[kBatch3dStages]) {
    const size_t n = (size_t)(p.X + kQP) * (p.Y + kQP) * (p.Z + kQP);
    if (n >= (1ull << 32))
        return set_error(CG_ERR_INVALID, "volume too large for the batched quad forward");
    if (!p.d_volQA) {
        int rc = CG_OK;
        if (!try_malloc_or_oom((void **)&p.d_volQA, n * sizeof(float4), &rc) ||
            !try_malloc_or_oom((void **)&p.d_volQB, n * sizeof(float4), &rc)) {
            if (p.d_volQA) cudaFree(p.d_volQA);
            p.d_volQA = nullptr;
            return rc ? rc : set_error(CG_ERR_NOMEM, "no room for a batched problem's quads");
        }
    }
    if (int rc = ensure_plan3d_scratch(p, false, true)) return rc;
    if (!p.reads_quads())
        return set_error(CG_ERR_NOMEM, "no room for a batched problem's projection quads");
    const int tex_warps = p.algo_fwd == 5 ? p.fwd_tex_warps : 0;
    if (tex_warps > 0)
        if (int rc = ensure_volume_texture3(p)) return rc;

    Prob3d r{};
    r.vol = vol, r.sino = sino;
    r.QA = p.d_volQA, r.QB = p.d_volQB;
    r.forg = p.d_forg, r.fdu = p.d_fdu, r.fdv = p.d_fdv, r.fsrc = p.d_fsrc;
    r.tex = tex_warps > 0 ? p.tex3 : 0;
    r.tex_warps = tex_warps, r.exact_t = p.exact_t ? 1 : 0;
    r.X = p.X, r.Y = p.Y, r.Z = p.Z, r.U = p.U, r.V = p.V, r.P = p.nangles;
    r.utiles = ceil_div(p.U, 32);
    r.sinoQ = p.d_sinoQ;
    r.axial = p.runs_axial() ? 1 : 0;
    // the single-problem launchers' constants, in the same FP32 operations
    const float zplane = p.DSO - p.DSD;
    const float hu = (float)(p.U / 2), hv = (float)(p.V / 2);
    if (r.axial) {
        // per view: p0 = (a0, a1, a2, a9), p1 = (a3, a4, a5, a6), p2 = (a7, a8)
        const int P = p.nangles;
        std::vector<float> h((size_t)P * 10);
        for (int j = 0; j < P; ++j) {
            const float *a = p.ax_views.data() + (size_t)j * 10;
            float *p0 = h.data() + (size_t)j * 4, *p1 = h.data() + (size_t)(P + j) * 4;
            float *p2 = h.data() + (size_t)P * 8 + (size_t)j * 2;
            p0[0] = a[0], p0[1] = a[1], p0[2] = a[2], p0[3] = a[9];
            p1[0] = a[3], p1[1] = a[4], p1[2] = a[5], p1[3] = a[6];
            p2[0] = a[7], p2[1] = a[8];
        }
        CG_TRY_CUDA(cudaMemcpy(ax, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
        r.ax0 = reinterpret_cast<const float4 *>(ax);
        r.ax1 = r.ax0 + P;
        r.ax2 = reinterpret_cast<const float2 *>(r.ax1 + P);
        r.num = zplane - p.bsrc[2];
        r.su = p.bsrc[0] + hu - 0.5f, r.sv = p.bsrc[1] + hv - 0.5f;
        r.tiles_x = ceil_div(p.X, 32), r.tiles_y = ceil_div(p.Y, 8), r.tiles_z = ceil_div(p.Z, 8);
    } else {
        r.borg = p.d_borg, r.bdx = p.d_bdx, r.bdy = p.d_bdy, r.bdz = p.d_bdz;
        r.bsx = p.bsrc[0], r.bsy = p.bsrc[1], r.bsz = p.bsrc[2];
        r.zplane = zplane, r.hu = hu, r.hv = hv;
        r.tiles_x = ceil_div(p.X, 32), r.tiles_y = ceil_div(p.Y, 8), r.tiles_z = ceil_div(p.Z, kBZ);
    }
    *q = r;

    const long long bricks = (long long)ceil_div(r.tiles_x, 2) * ceil_div(r.tiles_y, 8) *
                             ceil_div(r.tiles_z, 8) * 128;
    const long long elems = (long long)(p.X + 2 * kP3) * (p.Y + 2 * kP3) * (p.Z + 2 * kP3);
    const long long b[kBatch3dStages] = {
        ceil_div((long long)n, 256),
        (long long)ceil_div(p.Z + kQP, 32) * ceil_div(p.X + kQP, 32) * (p.Y + kQP),
        (long long)r.utiles * p.nangles * ceil_div(p.V, 8),
        ceil_div((long long)(p.U + 2 * kP3) * (p.V + 2 * kP3) * p.nangles, 256),
        r.axial ? bricks : 0,
        r.axial ? 0 : bricks,
        ceil_div(2 * elems, 256),
        (long long)r.utiles * p.nangles * ceil_div(p.V, 8),
        ceil_div((long long)p.X * p.Y * p.Z, 256)};
    for (int st = 0; st < kBatch3dStages; ++st) {
        if (b[st] >= (1ll << 31)) return set_error(CG_ERR_INVALID, "problem too large for a batch");
        blocks[st] = (int)b[st];
    }
    return CG_OK;
}

int launch_batch3d_forward(const Prob3d *d_probs, const int *starts,
                           const int totals[kBatch3dStages], int count, cudaStream_t s) {
    const int n1 = count + 1;
    if (totals[0] > 0) {
        k_batch3d_qa<<<totals[0], 256, 0, s>>>(d_probs, starts, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (totals[1] > 0) {
        k_batch3d_qb<<<totals[1], dim3(32, 8), 0, s>>>(d_probs, starts + n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (totals[2] > 0) {
        k_batch3d_fwd<<<totals[2], 256, 0, s>>>(d_probs, starts + 2 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    return CG_OK;
}

int launch_batch3d_backward(const Prob3d *d_probs, const int *starts,
                            const int totals[kBatch3dStages], int count, cudaStream_t s) {
    const int n1 = count + 1;
    if (totals[3] > 0) {
        k_batch3d_relayout_sino<<<totals[3], 256, 0, s>>>(d_probs, starts + 3 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (totals[4] > 0) {
        k_batch3d_bwd_ax<8><<<totals[4], 256, 0, s>>>(d_probs, starts + 4 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    if (totals[5] > 0) {
        k_batch3d_bwd<<<totals[5], dim3(32, 8), 0, s>>>(d_probs, starts + 5 * n1, count);
        CG_TRY_CUDA(cudaGetLastError());
    }
    return CG_OK;
}

}  // namespace cg
