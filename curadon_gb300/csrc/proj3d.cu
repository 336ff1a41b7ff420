// proj3d.cu -- 3D cone-beam projection kernels for sm_103a.
//
// Data layout in HBM (all float32, per plan, allocated on first use):
//   volA  (Z+2P)(Y+2P)(X+2P) float2, pairs along x: (v[z][y][x], v[z][y][x+1])
//   volB  (X+2P)(Y+2P)(Z+2P) float2, pairs along z: (v[z][y][x], v[z+1][y][x])
//   sinoP nangles (V+2P)(U+2P) float2, pairs along u as (s[u], s[u+1] - s[u])
// with P = kPad zero texels on every face.  A warp handles 32 adjacent
// detector cells; for a circular orbit about y those cells are spread along
// x when the ray runs along z and along z when it runs along x, so each ray
// samples the copy whose contiguous axis is the one its warp spreads over,
// and four 8-byte loads gather the eight texels of a trilinear sample.
#include <cfloat>

#include "common.cuh"

namespace cg {
namespace {

constexpr int kP3 = kPad;

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
    A[idx] = make_float2(t0, t1);
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
                make_float2(tile[tz][i], tile[tz + 1][i]);
    }
    (void)PX;
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

// ------------------------------------------------------------ forward

// One thread per ray (u, v, view), the reference's ray set-up and float
// t-loop (forward_3d.hpp:56-93, intersection.h:12-28): the sample points are
// the reference's exactly up to FMA contraction; trilinear filtering is FP32
// in registers.  Rays that miss the box [-1, N+1]^3 write nothing.
__global__ void __launch_bounds__(256)
    k_fwd3d(const float2 *__restrict__ A, const float2 *__restrict__ B, float *__restrict__ sino,
            const float4 *__restrict__ torg, const float4 *__restrict__ tdu,
            const float4 *__restrict__ tdv, const float4 *__restrict__ tsrc, int X, int Y, int Z,
            int U, int V) {
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
    const float amax = (float)Na, bmax = (float)Y, cmax = (float)Nc;
    const float lo = -(float)kP3;

    float acc = 0.f;
    float t = tmin;
    for (int k = 0; k <= nsteps + 1; ++k) {
        if (!(t <= tmax)) break;
        const float pa_ = fmaf(da, t, sa), pb_ = fmaf(dy, t, s.y), pc_ = fmaf(dc, t, sc);
        // texture coordinate p + 0.5 filtered at (p + 0.5) - 0.5 = p
        const float fa = fminf(fmaxf(floorf(pa_), lo), amax);
        const float fb = fminf(fmaxf(floorf(pb_), lo), bmax);
        const float fc = fminf(fmaxf(floorf(pc_), lo), cmax);
        const float wa = pa_ - fa, wb = pb_ - fb, wc = pc_ - fc;
        const float2 *p00 =
            L + ((size_t)((int)fc + kP3) * pb + ((int)fb + kP3)) * pa + ((int)fa + kP3);
        const float2 t00 = __ldg(p00);
        const float2 t10 = __ldg(p00 + pa);
        const float2 t01 = __ldg(p00 + (size_t)pa * pb);
        const float2 t11 = __ldg(p00 + (size_t)pa * pb + pa);
        const float l00 = fmaf(wa, t00.y - t00.x, t00.x);
        const float l10 = fmaf(wa, t10.y - t10.x, t10.x);
        const float l01 = fmaf(wa, t01.y - t01.x, t01.x);
        const float l11 = fmaf(wa, t11.y - t11.x, t11.x);
        const float m0 = fmaf(wb, l10 - l00, l00);
        const float m1 = fmaf(wb, l11 - l01, l01);
        acc += fmaf(wc, m1 - m0, m0);
        t += h;
    }
    sino[((size_t)view * V + iv) * U + iu] = acc;
}

// ------------------------------------------------------------ backward

constexpr int kBZ = 8;         // voxels per thread along z
constexpr int kBViews = 64;    // view tables staged per pass

struct BwdTab {
    float4 o, dx, dy, dz;
};

// Block = 32 (x) x 8 (y) threads, each with a run of kBZ voxels along z.
// Blocks are visited brick by brick (2 x 8 x 8 tiles) so that the blocks
// resident at one time cover a compact region of the volume and share the
// detector footprint they read from L2.  Per voxel and view: the reference's
// ray/plane intersection (backward_3d.hpp:78-94) -- the ray direction is
// stepped along z from the run's first voxel -- then a bilinear sample of the
// difference-encoded pair-packed projection in two 8-byte loads and three
// FMAs, accumulated in registers; the volume is read and written once.
__global__ void __launch_bounds__(256)
    k_bwd3d(float *__restrict__ vol, const float2 *__restrict__ S,
            const float4 *__restrict__ torg, const float4 *__restrict__ tdx,
            const float4 *__restrict__ tdy, const float4 *__restrict__ tdz, float srcx,
            float srcy, float srcz, float zplane, float hu, float hv, int X, int Y, int Z, int U,
            int V, int nangles, int tiles_x, int tiles_y, int tiles_z) {
    __shared__ BwdTab stab[kBViews];
    // brick-ordered tile index
    constexpr int BX = 2, BY = 8, BZ = 8;
    const int bricks_x = (tiles_x + BX - 1) / BX, bricks_y = (tiles_y + BY - 1) / BY;
    const int lin = blockIdx.x;
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
#pragma unroll
            for (int k = 0; k < kBZ; ++k) {
                const float t = __fdividef(num, dirz);
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
    if (!tile_ok || x >= X || y >= Y) return;
#pragma unroll
    for (int k = 0; k < kBZ; ++k) {
        const int z = z0 + k;
        if (z < Z) vol[((size_t)z * Y + y) * X + x] += acc[k];
    }
}

}  // namespace

// ------------------------------------------------------------ launchers

int ensure_plan3d_scratch(Plan3d &p, bool fwd, bool bwd) {
    if (fwd && !p.d_volA) {
        const size_t n = (size_t)(p.X + 2 * kP3) * (p.Y + 2 * kP3) * (p.Z + 2 * kP3);
        CG_TRY_CUDA(cudaMalloc(&p.d_volA, n * sizeof(float2)));
        CG_TRY_CUDA(cudaMalloc(&p.d_volB, n * sizeof(float2)));
        p.volA_elems = p.volB_elems = n;
    }
    if (bwd && !p.d_sinoP) {
        const size_t n = (size_t)(p.U + 2 * kP3) * (p.V + 2 * kP3) * p.nangles;
        CG_TRY_CUDA(cudaMalloc(&p.d_sinoP, n * sizeof(float2)));
        p.sinoP_elems = n;
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
                                         p.d_fsrc, p.X, p.Y, p.Z, p.U, p.V);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_backward3d(const Plan3d &p, float *vol, const float *sino, cudaStream_t s) {
    {
        const long long n = (long long)p.sinoP_elems;
        k_relayout_sino3d<<<ceil_div(n, 256), 256, 0, s>>>(sino, p.U, p.V, p.nangles, p.d_sinoP);
        CG_TRY_CUDA(cudaGetLastError());
    }
    const int tiles_x = ceil_div(p.X, 32), tiles_y = ceil_div(p.Y, 8), tiles_z = ceil_div(p.Z, kBZ);
    const int bricks = ceil_div(tiles_x, 2) * ceil_div(tiles_y, 8) * ceil_div(tiles_z, 8);
    const float zplane = p.DSO - p.DSD;
    const float hu = (float)(p.U / 2), hv = (float)(p.V / 2);
    k_bwd3d<<<bricks * 128, dim3(32, 8), 0, s>>>(
        vol, p.d_sinoP, p.d_borg, p.d_bdx, p.d_bdy, p.d_bdz, p.bsrc[0], p.bsrc[1], p.bsrc[2],
        zplane, hu, hv, p.X, p.Y, p.Z, p.U, p.V, p.nangles, tiles_x, tiles_y, tiles_z);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
