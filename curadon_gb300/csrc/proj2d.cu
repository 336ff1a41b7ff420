// proj2d.cu -- 2D fan-beam projection kernels for sm_103a.
//
// Data layout in HBM (all float32, per plan):
//   layA  (H+2P) rows x pitchA float2: layA[y][x] = (v[y][x], v[y][x+1] - v[y][x])
//   layB  (W+2P) rows x pitchB float2: layB[x][y] = (v[y][x], v[y+1][x] - v[y][x])
//   sinoP nangles rows x (det+2P) float2: sinoP[a][k] = (s[a][k], s[a][k+1] - s[a][k])
// with P = kPad texels of zeros around every edge (pitches rounded up to an
// even number of pairs so rows start on 16 bytes).  One 8-byte load then
// returns what a linear filter needs along the contiguous axis (the value and
// the difference to its neighbour, so the lerp is a single FMA), and a
// warp of adjacent detector cells (forward) or adjacent pixels (backward)
// reads consecutive addresses whatever the view angle: rays that advance
// along y read layA, rays that advance along x read the transposed layB.
// Interpolation is FP32 in registers (no texture unit); clamping a texel
// index into the zero padding reproduces cudaAddressModeBorder.
#include <algorithm>
#include <cfloat>
#include <climits>

#include "common.cuh"

namespace cg {
namespace {

// ------------------------------------------------------------ plan tables

// Clockwise rotation of v by (cs, sn) about the origin, minus t, as
// geometry::rotate (rotation.hpp:51-61) evaluates it when the reference's
// plan precompute is compiled: x = fma(v.x, cs, v.y sn) - t.x (the sum of
// two products fuses the first), y = fma(v.y, cs, -(v.x sn)) - t.y (the
// negated product becomes a subtraction that fuses the other).  Written out
// with fmaf so the roundings do not depend on how the compiler contracts
// this call site; checked bit for bit against the reference's tables.
__device__ __forceinline__ float2 rotate_minus(float2 v, float cs, float sn, float2 t) {
    return make_float2(fmaf(v.x, cs, v.y * sn) - t.x, fmaf(v.y, cs, -(v.x * sn)) - t.y);
}

// Per-view tables in voxel-index units, evaluated in FP32 with __cosf/__sinf
// in the order plan_2d::precompute uses (plan_2d.hpp:189-241, functors
// :17-80): the per-cell step is the difference of two rotated detector cells,
// so its rounding is amplified by the cell index and must match the
// reference's exactly for drop-in results at large detectors.
__global__ void k_plan2d_tables(int n, const float *__restrict__ ang,
                                const float *__restrict__ DSO, const float *__restrict__ DSD,
                                float det_ext, float ds, float doff, float sx, float sy,
                                float ox, float oy, float extx, float exty, float2 *src,
                                float2 *u0, float2 *du, float4 *bmeta, float4 *bproj) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = ang[i], dso = DSO[i], dsd = DSD[i];
    const float dod = dsd - dso;
    const float2 cell0 = make_float2(-det_ext / 2.f + ds * .5f, -dod);
    const float2 cell1 = make_float2(-det_ext / 2.f + ds * 1.5f, -dod);
    const float cs = __cosf(a), sn = __sinf(a);
    const float2 s = rotate_minus(make_float2(doff, dso), cs, sn, make_float2(0.f, 0.f));
    float2 o = rotate_minus(cell0, cs, sn, s);
    o = make_float2(o.x / sx, o.y / sy);
    float2 d = rotate_minus(cell1, cs, sn, s);
    d = make_float2(d.x / sx, d.y / sy);
    d = make_float2(d.x - o.x, d.y - o.y);
    const float2 ext = make_float2(0.5f * extx, 0.5f * exty);
    src[i] = make_float2((s.x - ox + ext.x) / sx, (s.y - oy + ext.y) / sy);
    u0[i] = o;
    du[i] = d;
    // (-sin, cos, DSD, DSO) as the backprojector's shared table
    // (backward_2d.hpp:45-55), with the same intrinsics.
    bmeta[i] = make_float4(-__sinf(a), __cosf(a), dsd, dso);
    // the same map as a projective table: den = (x' + DSO) / DSD, so that
    // w = 1 / den, and yi = (cos X - sin Y) / ds, so that u = yi w + det/2
    const float rd = 1.0f / dsd, rs = 1.0f / ds;
    bproj[i] = make_float4(-sn * rd, -cs * rd, dso * rd, 0.f);
    bproj[n + i] = make_float4(cs * rs, -sn * rs, 0.f, 0.f);
}

// ------------------------------------------------------------ re-layouts

constexpr int kTile = 32;

// Writes layA and layB for the 32 x 32 tile (bx, by) of padded texel space.
// ABS: the pairs (v[c] - (c - C) d[c], d[c]) with C = W / 2 (layA) or H / 2
// (layB), so that the linear sample at column coordinate p is e + (p - C) d
// with no fraction to form (the chunked forward's absolute-position form).
template <bool ABS = false>
__device__ __forceinline__ void relayout2d_tile(const float *__restrict__ vol, int W, int H,
                                                float2 *__restrict__ A, float2 *__restrict__ B,
                                                int pa, int pb, int bx, int by) {
    __shared__ float tile[kTile + 1][kTile + 1];
    const int x0 = bx * kTile - kPad, y0 = by * kTile - kPad;
    for (int j = threadIdx.y; j < kTile + 1; j += blockDim.y)
        for (int i = threadIdx.x; i < kTile + 1; i += blockDim.x) {
            const int x = x0 + i, y = y0 + j;
            tile[j][i] = (x >= 0 && x < W && y >= 0 && y < H) ? vol[(size_t)y * W + x] : 0.f;
        }
    __syncthreads();
    const int tx = threadIdx.x;
    for (int j = threadIdx.y; j < kTile; j += blockDim.y) {
        const int y = y0 + j, x = x0 + tx;
        if (y < H + kPad && x < W + kPad) {
            const float v = tile[j][tx], d = tile[j][tx + 1] - v;
            A[(size_t)(y + kPad) * pa + (x + kPad)] =
                make_float2(ABS ? fmaf(-(float)(x - W / 2), d, v) : v, d);
        }
    }
    for (int i = threadIdx.y; i < kTile; i += blockDim.y) {
        const int x = x0 + i, y = y0 + tx;
        if (x < W + kPad && y < H + kPad) {
            const float v = tile[tx][i], d = tile[tx + 1][i] - v;
            B[(size_t)(x + kPad) * pb + (y + kPad)] =
                make_float2(ABS ? fmaf(-(float)(y - H / 2), d, v) : v, d);
        }
    }
}

template <bool ABS>
__global__ void __launch_bounds__(256)
    k_relayout2d(const float *__restrict__ vol, int W, int H, float2 *__restrict__ A,
                 float2 *__restrict__ B, int pa, int pb) {
    relayout2d_tile<ABS>(vol, W, H, A, B, pa, pb, blockIdx.x, blockIdx.y);
}

// ABS: (t[k] - (k - det / 2) d[k], d[k]), the staged backprojector's
// absolute-position form (a sample at cell coordinate u is e + (u - det / 2) d).
template <bool ABS = false>
__device__ __forceinline__ void relayout_sino2d_elem(const float *__restrict__ sino, int det,
                                                     int nangles, float2 *__restrict__ S,
                                                     long long idx) {
    const int pitch = det + 2 * kPad;
    if (idx >= (long long)pitch * nangles) return;
    const int a = (int)(idx / pitch);
    const int k = (int)(idx % pitch) - kPad;
    const float *row = sino + (size_t)a * det;
    const float t0 = (k >= 0 && k < det) ? row[k] : 0.f;
    const float t1 = (k + 1 >= 0 && k + 1 < det) ? row[k + 1] : 0.f;
    const float d = t1 - t0;
    S[idx] = make_float2(ABS ? fmaf(-(float)(k - det / 2), d, t0) : t0, d);
}

template <bool ABS>
__global__ void k_relayout_sino2d(const float *__restrict__ sino, int det, int nangles,
                                  float2 *__restrict__ S) {
    relayout_sino2d_elem<ABS>(sino, det, nangles, S,
                              (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------------------------ forward

// One thread per ray (detector cell u, view): the reference's ray set-up
// (forward_2d.hpp:52-68, intersection.h:31-46) in the same FP32 operations,
// then rint(max|rd|) unit steps along the dominant axis.  Along that axis the
// step is exactly +-1, so the row index advances by one and the vertical
// filter weight stays fixed; the two row sums are blended once at the end.
__device__ __forceinline__ void fwd2d_ray(const float2 *__restrict__ layA,
                                          const float2 *__restrict__ layB,
                                          float *__restrict__ sino,
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
    float *out = sino + (size_t)view * det + u;
    if ((double)tmin > (double)tmax - 1e-6) {
        *out = 0.f;
        return;
    }
    const float rox = fmaf(dx, tmin, s.x), roy = fmaf(dy, tmin, s.y);
    const float tl = tmax - tmin;
    const float rdx = dx * tl, rdy = dy * tl;
    const float m = fmaxf(fabsf(rdx), fabsf(rdy));
    int n = __float2int_rn(m);
    const float vx = rdx / m, vy = rdy / m;

    const bool ymajor = fabsf(rdy) >= fabsf(rdx);
    float p = (ymajor ? rox : roy) - 0.5f;
    const float vp = ymajor ? vx : vy;
    const float q = (ymajor ? roy : rox) - 0.5f;
    const int sq = ((ymajor ? vy : vx) > 0.f) ? 1 : -1;
    const float2 *lay = ymajor ? layA : layB;
    const int pitch = ymajor ? pa : pb;
    const float pmax = (float)(ymajor ? W : H);
    const int qmax = ymajor ? H : W;

    const float qf = floorf(q);
    const float fq = q - qf;
    const int iq = (int)fminf(fmaxf(qf, -(float)kPad), (float)qmax);
    n = min(n, sq > 0 ? qmax - iq + 1 : iq + kPad + 1);
    const float2 *row = lay + (size_t)(iq + kPad) * pitch + kPad;
    const long long rstep = (long long)sq * pitch;

    float acc_lo = 0.f, acc_hi = 0.f;
#pragma unroll 4
    for (int j = 0; j < n; ++j) {
        const float pf = fminf(fmaxf(floorf(p), -(float)kPad), pmax);
        const float fp = p - pf;
        const int ip = (int)pf;
        const float2 lo = __ldg(row + ip);
        const float2 hi = __ldg(row + pitch + ip);
        acc_lo += fmaf(fp, lo.y, lo.x);
        acc_hi += fmaf(fp, hi.y, hi.x);
        p += vp;
        row += rstep;
    }
    const float acc = fmaf(fq, acc_hi - acc_lo, acc_lo);
    *out = acc * hypotf(vx * sx, vy * sy);
}

__global__ void __launch_bounds__(256)
    k_fwd2d(const float2 *__restrict__ layA, const float2 *__restrict__ layB,
            float *__restrict__ sino, const float2 *__restrict__ tsrc,
            const float2 *__restrict__ tu0, const float2 *__restrict__ tdu, int W, int H,
            int det, int nangles, float sx, float sy, int pa, int pb) {
    fwd2d_ray(layA, layB, sino, tsrc, tu0, tdu, W, H, det, nangles, sx, sy, pa, pb,
              blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

// ------------------------------------------------------------ forward, shared ray set-up

// Ray set-up of the chunked forward: the reference's FP32 sequence
// (forward_2d.hpp:52-68, intersection.h:31-46).  Returns false for a ray that
// misses the box.
struct FanRay {
    float p, vp, q, fq, nrm;
    int n, sq;
    bool ymajor;
};

__device__ __forceinline__ bool fan_ray(const float2 s, const float2 o, const float2 du, int u,
                                        int W, int H, float sx, float sy, FanRay &r) {
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
    if ((double)tmin > (double)tmax - 1e-6) return false;
    const float rox = fmaf(dx, tmin, s.x), roy = fmaf(dy, tmin, s.y);
    const float tl = tmax - tmin;
    const float rdx = dx * tl, rdy = dy * tl;
    const float m = fmaxf(fabsf(rdx), fabsf(rdy));
    const float vx = rdx / m, vy = rdy / m;
    r.n = __float2int_rn(m);
    r.ymajor = fabsf(rdy) >= fabsf(rdx);
    r.p = (r.ymajor ? rox : roy) - 0.5f;
    r.vp = r.ymajor ? vx : vy;
    r.q = (r.ymajor ? roy : rox) - 0.5f;
    r.sq = ((r.ymajor ? vy : vx) > 0.f) ? 1 : -1;
    r.fq = r.q - floorf(r.q);
    r.nrm = hypotf(vx * sx, vy * sy);
    return true;
}

}  // namespace

__device__ unsigned long long g_wait_timeouts = 0;

int take_wait_timeouts(unsigned long long *count) {
    CG_TRY_CUDA(cudaMemcpyFromSymbol(count, g_wait_timeouts, sizeof(*count)));
    const unsigned long long zero = 0;
    CG_TRY_CUDA(cudaMemcpyToSymbol(g_wait_timeouts, &zero, sizeof(zero)));
    return CG_OK;
}

// True for the chunked forward's shapes that read the absolute-position
// layouts (relayout2d_tile<true>).
bool cslab_abs(int rows) { return rows == 474 || rows == 484; }

// True for the staged backprojector's variants that read the
// absolute-position sinogram pairs (relayout_sino2d_elem<true>).
bool bwd_abs(int min_blocks) { return min_blocks == 48 || min_blocks == 68; }

namespace {

// ------------------------------------------------------------ forward, chunked slab

constexpr int kCs2G = 4;             // views per bundle
constexpr int kCs2MaxChunks = 1024;  // chunk windows kept in shared memory

// Row-sum accumulation of one sample's two pairs.  Scalar: alo += lo.x +
// fp lo.y (same operations as the register forward).  Packed: the terms are
// kept apart, (sum lo.x, sum fp lo.y), one packed FP32 FMA per row.
template <bool PK>
struct RowAcc {
    float2 lo, hi;
    __device__ __forceinline__ void zero() { lo = hi = make_float2(0.f, 0.f); }
    __device__ __forceinline__ void add(float fp, float2 a, float2 b) {
        if constexpr (PK) {
            const float2 w = make_float2(1.f, fp);
            lo = __ffma2_rn(w, a, lo);
            hi = __ffma2_rn(w, b, hi);
        } else {
            lo.x += fmaf(fp, a.y, a.x);
            hi.x += fmaf(fp, b.y, b.x);
        }
    }
    __device__ __forceinline__ float sum_lo() const { return PK ? lo.x + lo.y : lo.x; }
    __device__ __forceinline__ float sum_hi() const { return PK ? hi.x + hi.y : hi.x; }
};

// Column index floor(p) - c0 clamped to [0, cmax] and the weight of the
// pair's second term: the fraction p - floor(p) for (v, d) pairs, p itself
// for the absolute-position form (e, d).
template <bool ABS>
__device__ __forceinline__ unsigned cs_column(float p, int c0, unsigned cmax, float &w) {
    if constexpr (ABS) {
        w = p;
        return min((unsigned)(__float2int_rd(p) - c0), cmax);
    } else {
        const float pf = floorf(p);
        w = p - pf;
        return min((unsigned)((int)pf - c0), cmax);
    }
}

// Bundle = kCs2G views x T adjacent detector cells x ray class (blockIdx.z:
// 0 = y-stepping rays on layA, 1 = x-stepping rays on layB); thread t owns
// cell u0 + t of every view.  The block walks its layout's rows in chunks of
// K.  A chunk's window -- the pair columns the bundle's rays can touch on its
// rows -- is bounded by lines through each view's source: a ray's column is
// linear in the row with slope b = dp/dq, and the rays of this class have
// |b| <= 1.  Over a detector interval on which dq keeps its sign b is
// monotone, so the slopes at the bundle's end cells clamped to [-1, 1] bound
// every ray of the class; where dq changes sign the bound is b = -1 .. 1.
// All windows are computed up front.  Windows are staged for rows r0 .. r0 +
// K (row stride S pairs) with 16-byte cp.async into two alternating buffers,
// the next chunk's copy running while the current chunk is sampled, one
// barrier per chunk.  Every ray then takes its samples of the chunk from
// shared memory: two 8-byte loads at fixed row offsets and two FMAs each
// (bound by the shared-memory data path, so the conversion unit's floor
// costs nothing here: the FP32-add floor measured slower).  Samples and
// weights are those of the register forward (the reference's positions; rays
// stepping towards smaller rows are summed in reverse), so the matched
// adjoint is this forward's transpose up to the order of summation.  A chunk
// whose window does not fit reads global memory.
// Waits (mbarrier tries) before a bulk copy counts as lost: far beyond any
// copy's latency; the kernel then records the timeout and goes on.
constexpr int kWaitTries = 1 << 22;

// One bundle (bx: cells, by: views, bz: ray class) of the chunked forward;
// the kernels below run it over a grid (one problem) or a work list (many).
template <int K, int S, int T, bool PK, bool REUSE = false, int VS = 1, int NG = kCs2G,
          int MB = 0, int MAP = 0, bool ABS = false, bool TMA = false>
__device__ __forceinline__ void cslab_bundle(const float2 *__restrict__ layA,
                                             const float2 *__restrict__ layB,
                                             float *__restrict__ sino,
                                             const float2 *__restrict__ tsrc,
                                             const float2 *__restrict__ tu0,
                                             const float2 *__restrict__ tdu, int W, int H, int det,
                                             int nangles, float sx, float sy, int pa, int pb,
                                             int bx, int by, int bz) {
    static_assert(S % 2 == 0, "rows of the window buffers must stay 16-byte aligned");
    constexpr int kBuf = (K + 1) * S;               // pairs per buffer
    extern __shared__ __align__(16) float2 cwin[];  // 2 buffers
    __shared__ float s_cor[2 * NG][2];               // column = a + b * row
    __shared__ int s_win[kCs2MaxChunks];             // (first column << 16) | width, or -1
    __shared__ int s_rmin, s_rmax;
    const bool cls_y = bz == 0;
    const float2 *lay = cls_y ? layA : layB;
    const int pitch = cls_y ? pa : pb;
    const int qmax = cls_y ? H : W;
    const int pmaxi = cls_y ? W : H;
    // VS = 2: 2T threads, each on 2 of the bundle's 4 views; a warp holds 16
    // adjacent cells of two views, so one shared load spans half the columns
    // of 32 adjacent cells (fewer bank conflicts)
    constexpr int NT = T * VS, GV = NG / VS;
    static_assert(VS == 1 || ((VS == 2 || VS == 4) && NG % VS == 0), "view split of 1, 2, 4");
    static_assert(2 * NG <= 32, "corner lanes within one warp");
    // VS > 1: a warp holds 16 adjacent cells x 2 view groups; cells advance
    // every 16 * VS threads
    // MAP = 1 (VS = 2): each half-warp holds 8 cells x 2 view groups, so the
    // 64-bit shared loads of one half span ~8 columns (no bank conflicts)
    // MAP = 2: the same lanes, views interleaved (group j takes views j, j + 2,
    // ...), so the two groups of a half-warp are one view apart, not NG / 2
    static_assert(MAP == 0 || VS == 2, "the half-warp map is for two threads per cell");
    const int cell = VS == 1 ? (int)threadIdx.x
                     : MAP >= 1 ? (int)((threadIdx.x >> 5) * 16 + (threadIdx.x & 7) +
                                        8 * ((threadIdx.x >> 4) & 1))
                                : (int)((threadIdx.x / (16 * VS)) * 16 + (threadIdx.x & 15));
    const int gb = VS == 1     ? 0
                   : MAP >= 1 ? (int)((threadIdx.x >> 3) & 1) * GV
                              : (int)((threadIdx.x >> 4) % VS) * GV;
    // bundle view of the thread's ray g
    auto bview = [&](int g) { return MAP == 2 ? gb / GV + g * VS : gb + g; };
    const int u0 = bx * T, v0 = by * NG;
    const int u = u0 + cell;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) s_rmin = INT_MAX, s_rmax = INT_MIN;
    __syncthreads();
    if (threadIdx.x < 2 * NG) {  // lanes 2g, 2g + 1: the end cells of view g
        const int view = min(v0 + (threadIdx.x >> 1), nangles - 1);
        const int cu = (threadIdx.x & 1) ? min(u0 + T - 1, det - 1) : u0;
        const float2 sv = tsrc[view], o = tu0[view], d = tdu[view];
        const float dx = fmaf(d.x, (float)cu, o.x), dy = fmaf(d.y, (float)cu, o.y);
        // column p (texel coordinate - 1/2) of the ray on row q (the same)
        const float dp = cls_y ? dx : dy, dq = cls_y ? dy : dx;
        const float sp = (cls_y ? sv.x : sv.y) - 0.5f, sq = (cls_y ? sv.y : sv.x) - 0.5f;
        constexpr unsigned kCorners = 2 * NG == 32 ? 0xffffffffu : (1u << (2 * NG)) - 1u;
        const float dq_other = __shfl_xor_sync(kCorners, dq, 1);
        const float b = (dq > 0.f) != (dq_other > 0.f) ? ((threadIdx.x & 1) ? 1.f : -1.f)
                                                        : fminf(fmaxf(dp / dq, -1.f), 1.f);
        s_cor[threadIdx.x][0] = sp - sq * b;
        s_cor[threadIdx.x][1] = b;
    }
    // ABS: columns are kept relative to C = pmaxi / 2 (the layout's pairs
    // are (v - (c - C) d, d)), a sample is e + p d with p the relative column
    const int ic = ABS ? pmaxi / 2 : 0;
    const float pc = (float)ic;
    // per ray: column at its first row (p), step per row (V), row sums
    float p[GV], V[GV];
    RowAcc<PK> acc[GV];
    int rlo[GV], len[GV];
    int my_min = INT_MAX, my_max = INT_MIN;
#pragma unroll
    for (int g = 0; g < GV; ++g) {
        const int view = v0 + bview(g);
        acc[g].zero(), len[g] = 0, rlo[g] = 0, p[g] = V[g] = 0.f;
        if (view >= nangles || u >= det) continue;
        FanRay r;
        if (!fan_ray(tsrc[view], tu0[view], tdu[view], u, W, H, sx, sy, r)) continue;
        if (r.ymajor != cls_y) continue;
        const int iq = (int)fminf(fmaxf(floorf(r.q), -(float)kPad), (float)qmax);
        const int n = min(r.n, r.sq > 0 ? qmax - iq + 1 : iq + kPad + 1);
        if (n <= 0) continue;
        const int lo = r.sq > 0 ? iq : iq - (n - 1);
        V[g] = r.sq > 0 ? r.vp : -r.vp;
        p[g] = (r.sq > 0 ? r.p : fmaf((float)(n - 1), r.vp, r.p)) - pc;
        rlo[g] = lo, len[g] = n;
        my_min = min(my_min, lo), my_max = max(my_max, lo + n - 1);
    }
    if (my_min <= my_max) {
        atomicMin(&s_rmin, my_min);
        atomicMax(&s_rmax, my_max);
    }
    __syncthreads();
    const int rmin = s_rmin, rmax = s_rmax;
    const int nch = rmin <= rmax ? (rmax - rmin) / K + 1 : 0;
    {
        for (int ci = threadIdx.x; ci < min(nch, kCs2MaxChunks); ci += NT) {
            const float ra = (float)(rmin + ci * K), rb = ra + (float)K;
            float lo = FLT_MAX, hi = -FLT_MAX;
#pragma unroll
            for (int c = 0; c < 2 * NG; ++c) {
                const float c0 = fmaf(s_cor[c][1], ra, s_cor[c][0]);
                const float c1 = fmaf(s_cor[c][1], rb, s_cor[c][0]);
                lo = fminf(lo, fminf(c0, c1));
                hi = fmaxf(hi, fmaxf(c0, c1));
            }
            int win = -1;
            if (lo > -1e6f && hi < 1e6f) {
                // first column even (16-byte aligned rows), even width
                const int a0 = max((int)floorf(lo) - 1, -kPad) & ~1;
                const int a1 = min((int)floorf(hi) + 1, pmaxi + 1);
                const int wx = (a1 - a0 + 2) & ~1;
                if (a1 >= a0 && wx <= S) win = ((a0 + kPad) << 16) | wx;
            }
            s_win[ci] = win;
        }
    }
    __syncthreads();

    // copies chunk ci's window into buffer `buf`
    auto stage = [&](int ci, int buf) {
        const int win = ci < kCs2MaxChunks ? s_win[ci] : -1;
        if (win < 0) return;
        const int c0 = win >> 16, wx = win & 0xffff, r0 = rmin + ci * K;
        float2 *base = cwin + buf * kBuf;
        for (int row = warp; row <= K; row += NT / 32) {
            const int q = min(r0 + row, qmax + 1);
            const float2 *src = lay + (size_t)(q + kPad) * pitch + c0;
            float2 *dst = base + row * S;
            for (int c = 2 * lane; c < wx; c += 64) {
                const unsigned d = (unsigned)__cvta_generic_to_shared(dst + c);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + c));
            }
        }
    };

    // TMA: the chunk's K + 1 window rows come by bulk copies of the tensor
    // memory access unit, one per row issued by lanes of warp 0, completed on
    // the buffer's mbarrier (one arrival carrying the bytes); the barrier at
    // the top of each chunk still guards the buffer being refilled
    __shared__ __align__(8) unsigned long long s_bar[2];
    const unsigned bar0 = (unsigned)__cvta_generic_to_shared(&s_bar[0]);
    auto stage_tma = [&](int ci, int buf) {
        const int win = ci < kCs2MaxChunks ? s_win[ci] : -1;
        if (win < 0 || warp != 0) return;
        const int c0 = win >> 16, wx = win & 0xffff, r0 = rmin + ci * K;
        const unsigned bar = bar0 + 8u * (unsigned)buf;
        const unsigned row_bytes = (unsigned)wx * (unsigned)sizeof(float2);
        if (lane == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bar, (unsigned)(K + 1) * row_bytes);
        }
        __syncwarp();
        const unsigned base = (unsigned)__cvta_generic_to_shared(cwin + buf * kBuf);
        for (int row = lane; row <= K; row += 32) {
            const int q = min(r0 + row, qmax + 1);
            bulk_copy_g2s(base + (unsigned)(row * S) * (unsigned)sizeof(float2),
                          lay + (size_t)(q + kPad) * pitch + c0, row_bytes, bar);
        }
    };
    // TMA bookkeeping, per thread: completed phases of each buffer's barrier
    // (mod 2), buffers whose copies it has not yet seen complete, and whether
    // one of its waits gave up.  A give-up stops the block at the next chunk
    // boundary (every thread learns it from the same barrier), so no further
    // copy is issued; before exit thread 0 waits, again bounded, for the
    // copies still outstanding.  The block's outputs are then not to be
    // trusted and the give-up is counted for cg_wait_timeouts.
    unsigned phases = 0, pending = 0;
    int gave_up = 0;
    auto staged = [&](int ci) { return ci < kCs2MaxChunks && s_win[ci] >= 0; };
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            mbar_init(bar0, 1);
            mbar_init(bar0 + 8u, 1);
            mbar_fence_init();
        }
        __syncthreads();
        if (nch > 0) {
            stage_tma(0, 0);
            if (staged(0)) pending |= 1u;
        }
    } else {
        if (nch > 0) stage(0, 0);
        asm volatile("cp.async.commit_group;\n" ::);
    }
    for (int ci = 0; ci < nch; ++ci) {
        if constexpr (TMA) {
            if (__syncthreads_or(gave_up)) break;
            if (ci + 1 < nch) {
                stage_tma(ci + 1, (ci + 1) & 1);
                if (staged(ci + 1)) pending |= 1u << ((ci + 1) & 1);
            }
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::);
            __syncthreads();
            if (ci + 1 < nch) stage(ci + 1, (ci + 1) & 1);
            asm volatile("cp.async.commit_group;\n" ::);
        }
        const int r0 = rmin + ci * K;
        const int win = ci < kCs2MaxChunks ? s_win[ci] : -1;
        if (TMA && win >= 0) {
            const int b = ci & 1;
            if (mbar_wait(bar0 + 8u * (unsigned)b, (phases >> b) & 1u, kWaitTries)) {
                phases ^= 1u << b;
                pending &= ~(1u << b);
            } else {
                gave_up = 1;
            }
        }
        if (win >= 0) {
            const int c0 = (win >> 16) - kPad, wx = win & 0xffff;
            const unsigned cmax = (unsigned)(wx - 1);
            const float2 *b0 = cwin + (ci & 1) * kBuf;
#pragma unroll
            for (int g = 0; g < GV; ++g) {
                const int rel = r0 - rlo[g];
                if (rel >= 0 && rel + K <= len[g]) {
                    // REUSE: row k's lower pair is row k-1's upper pair when the
                    // column did not change (|step| <= 1 column per row), so
                    // only the lanes whose column moved load it
                    unsigned c_prev = 0xffffffffu;
                    float2 hi_prev = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        float fp;
                        const unsigned c = cs_column<ABS>(p[g], c0 - ic, cmax, fp);
                        const float2 hi = b0[(k + 1) * S + c];
                        float2 lo;
                        if (REUSE && c == c_prev) lo = hi_prev;
                        else lo = b0[k * S + c];
                        acc[g].add(fp, lo, hi);
                        if (REUSE) c_prev = c, hi_prev = hi;
                        p[g] += V[g];
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        if ((unsigned)(rel + k) < (unsigned)len[g]) {
                            float fp;
                            const unsigned c = cs_column<ABS>(p[g], c0 - ic, cmax, fp);
                            const float2 lo = b0[k * S + c], hi = b0[(k + 1) * S + c];
                            acc[g].add(fp, lo, hi);
                            p[g] += V[g];
                        }
                    }
                }
            }
        } else {
            const unsigned gcap = (unsigned)(pmaxi + kPad);
#pragma unroll
            for (int g = 0; g < GV; ++g) {
                const int ra = max(r0, rlo[g]), rb = min(r0 + K - 1, rlo[g] + len[g] - 1);
                for (int r = ra; r <= rb; ++r) {
                    float fp;
                    const unsigned c = cs_column<ABS>(p[g], -kPad - ic, gcap, fp);
                    const float2 *rowp = lay + (size_t)(r + kPad) * pitch;
                    const float2 lo = __ldg(rowp + c), hi = __ldg(rowp + pitch + c);
                    acc[g].add(fp, lo, hi);
                    p[g] += V[g];
                }
            }
        }
    }
    if constexpr (!TMA) asm volatile("cp.async.wait_group 0;\n" ::);
    if constexpr (TMA) {
        if (__syncthreads_or(gave_up) && threadIdx.x == 0) {
            atomicAdd(&g_wait_timeouts, 1ull);
            for (int b = 0; b < 2; ++b)
                if ((pending >> b) & 1u) mbar_wait(bar0 + 8u * (unsigned)b, (phases >> b) & 1u, kWaitTries);
        }
    }

#pragma unroll
    for (int g = 0; g < GV; ++g) {
        const int view = v0 + bview(g);
        if (view >= nangles || u >= det) continue;
        FanRay r;
        float out;
        if (!fan_ray(tsrc[view], tu0[view], tdu[view], u, W, H, sx, sy, r)) {
            if (!cls_y) continue;
            out = 0.f;
        } else {
            if (r.ymajor != cls_y) continue;
            const float alo = acc[g].sum_lo(), ahi = acc[g].sum_hi();
            out = fmaf(r.fq, ahi - alo, alo) * r.nrm;
        }
        sino[(size_t)view * det + u] = out;
    }
}

template <int K, int S, int T, bool PK, bool REUSE = false, int VS = 1, int NG = kCs2G,
          int MB = 0, int MAP = 0, bool ABS = false, bool TMA = false>
__global__ void __launch_bounds__(T * VS, MB)
    k_fwd2d_cslab(const float2 *__restrict__ layA, const float2 *__restrict__ layB,
                  float *__restrict__ sino, const float2 *__restrict__ tsrc,
                  const float2 *__restrict__ tu0, const float2 *__restrict__ tdu, int W, int H,
                  int det, int nangles, float sx, float sy, int pa, int pb) {
    cslab_bundle<K, S, T, PK, REUSE, VS, NG, MB, MAP, ABS, TMA>(
        layA, layB, sino, tsrc, tu0, tdu, W, H, det, nangles, sx, sy, pa, pb, blockIdx.x,
        blockIdx.y, blockIdx.z);
}

}  // namespace

int launch_forward2d_cslab(const Plan2d &p, float *sino, cudaStream_t s, int rows, int v0,
                           int nv) {
    // views [v0, v0 + nv): the kernel sees offset tables and sinogram rows
    if (nv < 0) nv = p.nangles - v0;
    if (nv <= 0) return CG_OK;
    const int ng = 8;  // views per bundle of the compiled shapes
    const int groups = ceil_div(nv, ng);
    if (groups > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    if (std::max(p.pitchA(), p.pitchB()) >= 32768)
        return set_error(CG_ERR_INVALID, "volume too wide for the chunked forward");
    auto go = [&](auto kernel, int k, int stride, int cells, int vs = 1) -> int {
        const size_t smem = 2 * sizeof(float2) * (k + 1) * stride;
        if (int rc = ensure_smem_attr((const void *)kernel, (int)smem)) return rc;
        dim3 grid(ceil_div(p.det, cells), groups, 2);
        kernel<<<grid, cells * vs, smem, s>>>(p.d_layA, p.d_layB, sino + (size_t)v0 * p.det,
                                           p.d_src + v0, p.d_u0 + v0, p.d_du + v0, p.W, p.H,
                                           p.det, nv, p.sx, p.sy, p.pitchA(), p.pitchB());
        CG_TRY_CUDA(cudaGetLastError());
        return CG_OK;
    };
    // the default (484) and the autotuner's other candidates (474: the same
    // staged by per-lane cp.async, 6 % slower at n=2048; 443: (v, d) pairs,
    // pair reuse, view groups four views apart, 30 % slower)
    switch (rows) {
        case 443: return go(k_fwd2d_cslab<16, 256, 128, true, true, 2, 8, 3, 1>, 16, 256, 128, 2);
        case 474: return go(k_fwd2d_cslab<16, 256, 128, true, false, 2, 8, 3, 2, true>, 16, 256, 128, 2);
        case 484: return go(k_fwd2d_cslab<16, 256, 128, true, false, 2, 8, 3, 2, true, true>, 16, 256, 128, 2);
        default: return set_error(CG_ERR_INVALID, "unknown chunk shape");
    }
}

namespace {

// ------------------------------------------------------------ backward

constexpr int kBwdRows = 4;        // pixels per thread, 8 rows apart
constexpr int kBwdViews = 256;     // per-view table entries staged per pass

// One thread per 4 pixels of a column; a 32 x 32 pixel tile per block.  Per
// view: x' = -s X - c Y, w = DSD / (x' + DSO), u = w (c X - s Y) / ds + det/2
// in the reference's FP32 operations (backward_2d.hpp:61-96), a linear
// sample of the pair-packed sinogram row, acc += sample * w; finally the
// volume gets acc / ds added (:99).
__global__ void __launch_bounds__(256)
    k_bwd2d(float *__restrict__ vol, const float2 *__restrict__ S,
            const float4 *__restrict__ meta, int W, int H, int det, int nangles, float sx,
            float sy, float ox, float oy, float ds) {
    __shared__ float4 smeta[kBwdViews];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y0 = blockIdx.y * 32 + threadIdx.y;
    const float ex = (float)W / 2.0f, ey = (float)H / 2.0f, ed = (float)det / 2.0f;
    const float inv = __fdividef(1.0f, ds);
    const float X = ((float)x - ex) * sx + ox + 0.5f;
    const float SX = X * inv;
    float Y[kBwdRows], SY[kBwdRows], acc[kBwdRows];
#pragma unroll
    for (int r = 0; r < kBwdRows; ++r) {
        Y[r] = ((float)(y0 + 8 * r) - ey) * sy + oy + 0.5f;
        SY[r] = Y[r] * inv;
        acc[r] = 0.f;
    }
    const int pitch = det + 2 * kPad;
    const float kmax = (float)det;
    for (int v0 = 0; v0 < nangles; v0 += kBwdViews) {
        const int nv = min(kBwdViews, nangles - v0);
        __syncthreads();
        for (int i = tid; i < nv; i += 256) smeta[i] = meta[v0 + i];
        __syncthreads();
        const float2 *rowbase = S + (size_t)v0 * pitch + kPad;
#pragma unroll 2
        for (int j = 0; j < nv; ++j) {
            const float4 m = smeta[j];  // (-sin, cos, DSD, DSO)
            const float2 *row = rowbase + (size_t)j * pitch;
#pragma unroll
            for (int r = 0; r < kBwdRows; ++r) {
                const float xi = m.x * X - m.y * Y[r];
                const float yi = m.y * SX + m.x * SY[r];
                const float w = __fdividef(m.z, xi + m.w);
                const float ub = (w * yi + ed) - 0.5f;
                const float kf = fminf(fmaxf(floorf(ub), -(float)kPad), kmax);
                const float a = ub - kf;
                const float2 t = __ldg(row + (int)kf);
                acc[r] = fmaf(fmaf(a, t.y, t.x), w, acc[r]);
            }
        }
    }
    if (x < W) {
#pragma unroll
        for (int r = 0; r < kBwdRows; ++r) {
            const int y = y0 + 8 * r;
            if (y < H) vol[(size_t)y * W + x] += acc[r] * inv;
        }
    }
}

// ------------------------------------------------------------ backward, staged

constexpr int kSmRows = 8;    // pixels per thread, 8 rows apart: 32 x 64 tiles
constexpr int kSmViews = 32;  // views staged per pass
constexpr int kSmWin = 128;   // pairs of one view's row staged for a tile

// The backprojection with each tile's detector window in shared memory.
// Per pass of 32 views, threads 0..31 project the tile's four corner pixels
// (a projective map sends the tile to an interval bounded by its corners),
// the block stages that window of the difference-encoded pair row, and every
// pixel samples it there; a view whose window exceeds kSmWin pairs is read
// from global memory instead.  Per (pixel, view) the reference's quantities
// (backward_2d.hpp:61-96) come from the view's projective table
// (den, yi affine in the pixel's world position X, Y):
//   w = 1 / den = DSD / (x' + DSO),  u = yi w + det/2,
// with the per-view terms of each thread's column hoisted, then one
// reciprocal, one 8-byte shared load and two FMAs.  The same table describes
// an arbitrary per-view source / detector placement (vector geometry).
// ABS: the sinogram pairs are (e, d) = (t - (k - det / 2) d, d) and a sample
// at cell coordinate ub is e + (ub - det / 2) d: the lateral coordinate is
// formed relative to det / 2 and serves as the weight, no fraction.
// MAPQ: each warp covers 8 x 4 pixels (per row group) instead of 32 x 1, so
// a half-warp's 16 lateral coordinates span fewer cells of the window row
// (fewer shared-memory bank conflicts where the magnification is high).
// BULK: each view's window row (kSmWin + 2 pairs, started on a 16-byte
// boundary) comes by one bulk copy of the tensor memory access unit, issued
// by a lane of warp 0 and completed on an mbarrier; rows whose window
// reaches past the padded sinogram row are copied pair by pair with the
// index clamp as before.
// R: pixels per thread (rows 8 apart), so tiles of 32 x 8R pixels; every
// pixel's sum runs over the views in the same order whatever R, so results
// do not depend on it.
template <bool PK, bool MAGIC = false, int VU = 2, bool CPA = false, bool ABS = false,
          bool MAPQ = false, bool BULK = false, int R = kSmRows>
__device__ __forceinline__ void bwd2d_smem_tile(float *__restrict__ vol,
                                                const float2 *__restrict__ S,
                                                const float4 *__restrict__ proj, int W, int H,
                                                int det, int nangles, float sx, float sy, float ox,
                                                float oy, float ds, int bx, int by) {
    constexpr int kRow = BULK ? kSmWin + 2 : kSmWin;  // pairs per staged row
    static_assert(kRow * sizeof(float2) % 16 == 0, "bulk rows are multiples of 16 bytes");
    __shared__ __align__(16) float2 srow[kSmViews][kRow];
    __shared__ float4 sA[kSmViews], sB[kSmViews];
    __shared__ int skmin[kSmViews];
    __shared__ int sbulk[kSmViews];
    __shared__ __align__(8) unsigned long long s_bar;
    const unsigned bar = (unsigned)__cvta_generic_to_shared(&s_bar);
    unsigned phase = 0;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int xt = bx * 32, yt = by * (8 * R);
    const int x = xt + (MAPQ ? (int)((threadIdx.y & 3) * 8 + (threadIdx.x & 7)) : (int)threadIdx.x);
    const int y0 = yt + (MAPQ ? (int)((threadIdx.y >> 2) * 4 + (threadIdx.x >> 3)) : (int)threadIdx.y);
    const float ex = (float)W / 2.0f, ey = (float)H / 2.0f;
    const float edm = (float)det / 2.0f - 0.5f;
    // sampling offset and index shift: ub - C and floor(ub - C) + C
    const int cq = ABS ? det / 2 : 0;
    const float edq = edm - (float)cq;
    const float inv = __fdividef(1.0f, ds);
    const float X = ((float)x - ex) * sx + ox + 0.5f;
    // rows r and r + 1 of the thread's column as one pair (the packed loop's
    // operands and accumulators)
    float2 Y2[R / 2], acc2[R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
        Y2[i] = make_float2(((float)(y0 + 16 * i) - ey) * sy + oy + 0.5f,
                            ((float)(y0 + 16 * i + 8) - ey) * sy + oy + 0.5f);
        acc2[i] = make_float2(0.f, 0.f);
    }
    auto Yv = [&](int r) -> float { return (r & 1) ? Y2[r >> 1].y : Y2[r >> 1].x; };
    auto add = [&](int r, float v) {
        if (r & 1) acc2[r >> 1].y += v; else acc2[r >> 1].x += v;
    };
    auto fma_acc = [&](int r, float a, float b) {
        if (r & 1) acc2[r >> 1].y = fmaf(a, b, acc2[r >> 1].y);
        else acc2[r >> 1].x = fmaf(a, b, acc2[r >> 1].x);
    };
    const int pitch = det + 2 * kPad;
    if constexpr (BULK) {
        if (tid == 0) {
            mbar_init(bar, 1);
            mbar_fence_init();
        }
    }
    // BULK: a wait that gives up stops the tile at the next group of views
    // (every thread learns it from the same barrier), so no further copy is
    // issued; before exit thread 0 waits, again bounded, for the copies it
    // has not seen complete.  The tile's results are then not to be trusted
    // and the give-up is counted for cg_wait_timeouts.
    int gave_up = 0;
    for (int v0 = 0; v0 < nangles; v0 += kSmViews) {
        const int nv = min(kSmViews, nangles - v0);
        if constexpr (BULK) {
            if (__syncthreads_or(gave_up)) break;
        } else {
            __syncthreads();
        }
        if (tid < nv) {
            const float4 a = proj[v0 + tid], b = proj[nangles + v0 + tid];
            sA[tid] = a, sB[tid] = b;
            float lo = FLT_MAX, hi = -FLT_MAX, dmin = FLT_MAX;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float cX = ((float)(xt + (c & 1) * 31) - ex) * sx + ox + 0.5f;
                const float cY = ((float)(yt + (c >> 1) * (8 * R - 1)) - ey) * sy + oy + 0.5f;
                const float den = fmaf(a.y, cY, fmaf(a.x, cX, a.z));
                const float yi = fmaf(b.y, cY, fmaf(b.x, cX, b.z));
                const float ub = fmaf(__fdividef(1.0f, den), yi, edm);
                lo = fminf(lo, ub);
                hi = fmaxf(hi, ub);
                dmin = fminf(dmin, den);
            }
            // the window bound holds when the tile lies wholly in front of the
            // source (den > 0 at every corner, hence on the whole tile)
            int k0 = INT_MIN, bulk = 0;
            if (dmin > 0.f && lo >= -1e6f && hi <= 1e6f) {
                const int a0 = (int)floorf(lo) - 1, a1 = (int)floorf(hi) + 1;
                if (a1 - a0 + 1 <= kSmWin) {
                    if constexpr (BULK) {
                        // start one pair earlier where needed so that the first
                        // staged pair (element (v0 + tid) pitch + kPad + k0) is
                        // even, i.e. on 16 bytes; the window then spans
                        // [k0, k0 + kSmWin + 1]
                        const int par = (int)(((long long)(v0 + tid) * pitch) & 1);
                        k0 = a0 - ((a0 ^ par) & 1);
                        bulk = k0 >= -kPad && k0 + kRow <= det + kPad;
                    } else {
                        k0 = a0;
                    }
                }
            }
            skmin[tid] = k0;
            sbulk[tid] = bulk;
        }
        __syncthreads();
        if constexpr (BULK) {
            // warp 0: the bulk rows, one copy per lane, on the block's barrier
            if (tid < 32) {
                const bool mine = tid < nv && sbulk[tid];
                const unsigned nb = __popc(__ballot_sync(0xffffffffu, mine));
                if (tid == 0) {
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(bar, nb * (unsigned)(kRow * sizeof(float2)));
                }
                __syncwarp();
                if (mine) {
                    fence_proxy_async_smem();
                    bulk_copy_g2s((unsigned)__cvta_generic_to_shared(&srow[tid][0]),
                                  S + (size_t)(v0 + tid) * pitch + kPad + skmin[tid],
                                  (unsigned)(kRow * sizeof(float2)), bar);
                }
            }
            // every warp: the other rows pair by pair (warp w: rows w, w + 8, ...)
            const int w = tid >> 5, ln = tid & 31;
            for (int j = w; j < nv; j += 8) {
                const int k0 = skmin[j];
                if (k0 == INT_MIN || sbulk[j]) continue;
                for (int i = ln; i < kRow; i += 32) {
                    const int k = min(max(k0 + i, -kPad), det);
                    const unsigned d = (unsigned)__cvta_generic_to_shared(&srow[j][i]);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d),
                                 "l"(S + (size_t)(v0 + j) * pitch + kPad + k));
                }
            }
            asm volatile("cp.async.wait_all;\n" ::);
            if (mbar_wait(bar, phase, kWaitTries)) phase ^= 1u;
            else gave_up = 1;
        }
        for (int e = tid; !BULK && e < nv * kSmWin; e += 256) {
            const int j = e / kSmWin, i = e - j * kSmWin;
            const int k0 = skmin[j];
            if (k0 == INT_MIN) continue;
            const int k = min(max(k0 + i, -kPad), det);
            if constexpr (CPA) {
                // 8-byte asynchronous copy, no register round trip
                const unsigned d = (unsigned)__cvta_generic_to_shared(&srow[j][i]);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d),
                             "l"(S + (size_t)(v0 + j) * pitch + kPad + k));
            } else {
                srow[j][i] = S[(size_t)(v0 + j) * pitch + kPad + k];
            }
        }
        if constexpr (CPA) asm volatile("cp.async.wait_all;\n" ::);
        __syncthreads();
#pragma unroll VU
        for (int j = 0; j < nv; ++j) {
            const float4 a = sA[j], b = sB[j];
            const int k0 = skmin[j];
            const float A = fmaf(a.x, X, a.z), B = fmaf(b.x, X, b.z);
            if (k0 != INT_MIN) {
                const float2 *sr = srow[j];
                if constexpr (PK) {
                    // two rows per packed FP32 instruction (the same IEEE
                    // operations per row as the scalar loop below)
                    const float2 ay = make_float2(a.y, a.y), by = make_float2(b.y, b.y);
                    const float2 A2 = make_float2(A, A), B2 = make_float2(B, B);
                    const float2 e2 = make_float2(edq, edq);
#pragma unroll
                    for (int r = 0; r < R; r += 2) {
                        const float2 Yr = Y2[r >> 1];
                        const float2 den = __ffma2_rn(ay, Yr, A2);
                        const float2 yi = __ffma2_rn(by, Yr, B2);
                        const float2 w = make_float2(rcp_approx(den.x), rcp_approx(den.y));
                        const float2 ub = __ffma2_rn(w, yi, e2);
                        float2 f;
                        unsigned l0, l1;
                        if constexpr (MAGIC) {
                            // floor without the conversion unit: ub + 1.5 * 2^23
                            // rounded toward -inf is floor(ub) + 1.5 * 2^23 exactly
                            // (unit spacing there); |ub| >= 2^22 lands outside the
                            // window and is clamped.  f = ub + (1.5 * 2^23 - t).
                            const float2 M2 = make_float2(12582912.0f, 12582912.0f);
                            const float2 t = __fadd2_rd(ub, M2);
                            f = ABS ? ub
                                    : __fadd2_rn(ub, __ffma2_rn(t, make_float2(-1.f, -1.f), M2));
                            const unsigned base = 0x4B400000u + (unsigned)(k0 - cq);
                            l0 = min(__float_as_uint(t.x) - base, (unsigned)(kRow - 1));
                            l1 = min(__float_as_uint(t.y) - base, (unsigned)(kRow - 1));
                        } else {
                            const float2 kf = make_float2(floorf(ub.x), floorf(ub.y));
                            f = ABS ? ub : __fadd2_rn(ub, make_float2(-kf.x, -kf.y));
                            l0 = min((unsigned)((int)kf.x + cq - k0), (unsigned)(kRow - 1));
                            l1 = min((unsigned)((int)kf.y + cq - k0), (unsigned)(kRow - 1));
                        }
                        const float2 t0 = sr[l0], t1 = sr[l1];
                        const float2 v = make_float2(fmaf(f.x, t0.y, t0.x), fmaf(f.y, t1.y, t1.x));
                        acc2[r >> 1] = __ffma2_rn(v, w, acc2[r >> 1]);
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float den = fmaf(a.y, Yv(r), A);
                        const float yi = fmaf(b.y, Yv(r), B);
                        const float w = rcp_approx(den);
                        const float ub = fmaf(w, yi, edq);
                        const float kf = floorf(ub);
                        const float f = ABS ? ub : ub - kf;
                        const unsigned li =
                            min((unsigned)((int)kf + cq - k0), (unsigned)(kRow - 1));
                        const float2 t = sr[li];
                        fma_acc(r, fmaf(f, t.y, t.x), w);
                    }
                }
            } else {
                const float2 *row = S + (size_t)(v0 + j) * pitch;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const float den = fmaf(a.y, Yv(r), A);
                    const float yi = fmaf(b.y, Yv(r), B);
                    const float w = rcp_approx(den);
                    const float ub = fmaf(w, yi, edq);
                    const float kf = floorf(ub);
                    const float f = ABS ? ub : ub - kf;
                    const unsigned col =
                        min((unsigned)((int)kf + cq + kPad), (unsigned)(det + kPad));
                    const float2 t = __ldg(row + col);
                    fma_acc(r, fmaf(f, t.y, t.x), w);
                }
            }
        }
    }
    if constexpr (BULK) {
        if (__syncthreads_or(gave_up) && tid == 0) {
            atomicAdd(&g_wait_timeouts, 1ull);
            if (gave_up) mbar_wait(bar, phase, kWaitTries);
        }
    }
    if (x < W) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int y = y0 + 8 * r;
            const float a = (r & 1) ? acc2[r >> 1].y : acc2[r >> 1].x;
            if (y < H) vol[(size_t)y * W + x] += a * inv;
        }
    }
}

// The staged backprojection over the views' quarter-turn symmetry.  When
// view v + n/4 is view v turned by 90 degrees about the image centre (the
// same DSO / DSD; a circular orbit whose n views, n divisible by 4, are
// spaced evenly over a full turn) and the pixels are square and centred,
// view v + n/4 sees pixel R P = (y, W - 1 - x) exactly as view v sees
// P = (x, y): the same denominator, weight and detector coordinate.  Each
// block therefore takes a tile of the image's first quadrant and its three
// turned copies: per view v and pixel P one projective evaluation (two FMAs,
// a reciprocal, one FMA, the floor) serves the four (pixel, view) pairs
// (R^i P, v + i n/4), each of which adds its own view's sample at the same
// detector coordinate from its own staged window row, so per sample only
// the shared-memory load and the lerp remain.  The four rows of a view
// share one window (the turned tile projects to the same interval);
// kSymViews views per pass, 4 kSymViews rows staged by bulk copies on the
// block's mbarrier.  DIR = -1: view v + n/4 sees R^-1 P instead.  Every
// pixel still sums all n views, in the order v + i n/4, v = 0 .. n - 1.
// NV views per pass, windows of WIN pairs.
constexpr int kSymR = 4, kSymNV = 16, kSymWin = 80;
template <int R, int NV, int WIN>
__device__ __forceinline__ void bwd2d_sym_tile(float *__restrict__ vol,
                                               const float2 *__restrict__ S,
                                               const float4 *__restrict__ proj, int W, int det,
                                               int nangles, float sx, float ox, float ds,
                                               int dir, int bx, int by) {
    constexpr int kSymViews = NV;
    constexpr int kRow = WIN + 2;  // pairs per staged row
    constexpr int kRows = 4 * kSymViews;
    static_assert(kRows <= 256, "one thread per staged row");
    static_assert(kRows % 32 == 0, "warp 0 counts the bulk rows in whole-warp rounds");
    static_assert(kRow * sizeof(float2) % 16 == 0, "bulk rows are multiples of 16 bytes");
    __shared__ __align__(16) float2 srow[kRows][kRow];
    __shared__ float4 sA[kSymViews], sB[kSymViews];
    __shared__ int sa0[kSymViews];
    __shared__ int sshift[kRows], sbulk[kRows];
    __shared__ __align__(8) unsigned long long s_bar;
    const unsigned bar = (unsigned)__cvta_generic_to_shared(&s_bar);
    unsigned phase = 0;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int half = W / 2, q = nangles / 4;
    const int xt = bx * 32, yt = by * (8 * R);
    const int x = xt + (int)((threadIdx.y & 3) * 8 + (threadIdx.x & 7));
    const int y0 = yt + (int)((threadIdx.y >> 2) * 4 + (threadIdx.x >> 3));
    const float ex = (float)W / 2.0f;
    const float edm = (float)det / 2.0f - 0.5f;
    const int cq = det / 2;
    const float edq = edm - (float)cq;
    const float inv = __fdividef(1.0f, ds);
    const float X = ((float)x - ex) * sx + ox + 0.5f;
    float2 Y2[R / 2], acc[4][R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
        Y2[i] = make_float2(((float)(y0 + 16 * i) - ex) * sx + ox + 0.5f,
                            ((float)(y0 + 16 * i + 8) - ex) * sx + ox + 0.5f);
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k][i] = make_float2(0.f, 0.f);
    }
    const int pitch = det + 2 * kPad;
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    // a wait that gives up stops the tile at the next group of views, as in
    // bwd2d_smem_tile
    int gave_up = 0;
    for (int v0 = 0; v0 < nangles; v0 += kSymViews) {
        const int nv = min(kSymViews, nangles - v0);
        if (__syncthreads_or(gave_up)) break;
        if (tid < nv) {
            const float4 a = proj[v0 + tid], b = proj[nangles + v0 + tid];
            sA[tid] = a, sB[tid] = b;
            float lo = FLT_MAX, hi = -FLT_MAX, dmin = FLT_MAX;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float cX = ((float)(xt + (c & 1) * 31) - ex) * sx + ox + 0.5f;
                const float cY = ((float)(yt + (c >> 1) * (8 * R - 1)) - ex) * sx + ox + 0.5f;
                const float den = fmaf(a.y, cY, fmaf(a.x, cX, a.z));
                const float yi = fmaf(b.y, cY, fmaf(b.x, cX, b.z));
                const float ub = fmaf(__fdividef(1.0f, den), yi, edm);
                lo = fminf(lo, ub);
                hi = fmaxf(hi, ub);
                dmin = fminf(dmin, den);
            }
            int a0 = INT_MIN;
            if (dmin > 0.f && lo >= -1e6f && hi <= 1e6f) {
                const int l0 = (int)floorf(lo) - 1, l1 = (int)floorf(hi) + 1;
                if (l1 - l0 + 1 <= WIN) a0 = l0;
            }
            sa0[tid] = a0;
        }
        __syncthreads();
        // rows 4 j + i: view (v0 + j + i q) mod n, pairs from a0 (shift 0) or
        // a0 - 1 (shift 1) so that a bulk copy starts on 16 bytes
        if (tid < 4 * nv) {
            const int j = tid >> 2, i = tid & 3;
            const int a0 = sa0[j];
            int shift = 0, bulk = 0;
            if (a0 != INT_MIN) {
                const long long view = (v0 + j + (long long)i * q) % nangles;
                const int par = (int)((view * pitch + kPad + a0) & 1);
                bulk = a0 - par >= -kPad && a0 - par + kRow <= det + kPad;
                shift = bulk ? par : 0;  // rows copied pair by pair start at a0
            }
            sshift[tid] = shift;
            sbulk[tid] = bulk;
        }
        __syncthreads();
        if (tid < 32) {
            // every lane takes part in every round (kRows is a multiple of 32)
            unsigned nb = 0;
#pragma unroll
            for (int round = 0; round < kRows / 32; ++round) {
                const int rr = round * 32 + tid;
                nb += __popc(__ballot_sync(0xffffffffu, rr < 4 * nv && sbulk[rr]));
            }
            if (tid == 0) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(bar, nb * (unsigned)(kRow * sizeof(float2)));
            }
            __syncwarp();
        }
        __syncthreads();
        if (tid < kRows) {
            const bool mine = tid < 4 * nv && sbulk[tid];
            if (mine) {
                const int j = tid >> 2, i = tid & 3;
                const long long view = (v0 + j + (long long)i * q) % nangles;
                fence_proxy_async_smem();
                bulk_copy_g2s((unsigned)__cvta_generic_to_shared(&srow[tid][0]),
                              S + (size_t)view * pitch + kPad + sa0[j] - sshift[tid],
                              (unsigned)(kRow * sizeof(float2)), bar);
            }
        }
        // rows whose window reaches past the padded sinogram row: pair by pair,
        // clamped (shift 0)
        {
            const int w = tid >> 5, ln = tid & 31;
            for (int rr = w; rr < 4 * nv; rr += 8) {
                const int j = rr >> 2, i = rr & 3;
                const int a0 = sa0[j];
                if (a0 == INT_MIN || sbulk[rr]) continue;
                const long long view = (v0 + j + (long long)i * q) % nangles;
                for (int e = ln; e < kRow; e += 32) {
                    const int k = min(max(a0 + e, -kPad), det);
                    const unsigned d = (unsigned)__cvta_generic_to_shared(&srow[rr][e]);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d),
                                 "l"(S + (size_t)view * pitch + kPad + k));
                }
            }
        }
        asm volatile("cp.async.wait_all;\n" ::);
        if (mbar_wait(bar, phase, kWaitTries)) phase ^= 1u;
        else gave_up = 1;
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < nv; ++j) {
            const float4 a = sA[j], b = sB[j];
            const int a0 = sa0[j];
            const float A = fmaf(a.x, X, a.z), B = fmaf(b.x, X, b.z);
            const float2 ay = make_float2(a.y, a.y), by = make_float2(b.y, b.y);
            const float2 A2 = make_float2(A, A), B2 = make_float2(B, B);
            const float2 e2 = make_float2(edq, edq);
            if (a0 != INT_MIN) {
                const float2 *p[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) p[i] = &srow[4 * j + i][sshift[4 * j + i]];
                const unsigned base = 0x4B400000u + (unsigned)(a0 - cq);
#pragma unroll
                for (int r = 0; r < R; r += 2) {
                    const float2 Yr = Y2[r >> 1];
                    const float2 den = __ffma2_rn(ay, Yr, A2);
                    const float2 yi = __ffma2_rn(by, Yr, B2);
                    const float2 w = make_float2(rcp_approx(den.x), rcp_approx(den.y));
                    const float2 ub = __ffma2_rn(w, yi, e2);
                    const float2 M2 = make_float2(12582912.0f, 12582912.0f);
                    const float2 t = __fadd2_rd(ub, M2);
                    const unsigned l0 = min(__float_as_uint(t.x) - base, (unsigned)(kRow - 2));
                    const unsigned l1 = min(__float_as_uint(t.y) - base, (unsigned)(kRow - 2));
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float2 t0 = p[i][l0], t1 = p[i][l1];
                        const float2 v = make_float2(fmaf(ub.x, t0.y, t0.x),
                                                     fmaf(ub.y, t1.y, t1.x));
                        acc[i][r >> 1] = __ffma2_rn(v, w, acc[i][r >> 1]);
                    }
                }
            } else {
                // a window wider than kSmWin: the four rows from global memory
#pragma unroll
                for (int r = 0; r < R; r += 2) {
                    const float2 Yr = Y2[r >> 1];
                    const float2 den = __ffma2_rn(ay, Yr, A2);
                    const float2 yi = __ffma2_rn(by, Yr, B2);
                    const float2 w = make_float2(rcp_approx(den.x), rcp_approx(den.y));
                    const float2 ub = __ffma2_rn(w, yi, e2);
                    const unsigned c0 = min((unsigned)((int)floorf(ub.x) + cq + kPad),
                                            (unsigned)(det + kPad));
                    const unsigned c1 = min((unsigned)((int)floorf(ub.y) + cq + kPad),
                                            (unsigned)(det + kPad));
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const long long view = (v0 + j + (long long)i * q) % nangles;
                        const float2 *row = S + (size_t)view * pitch;
                        const float2 t0 = __ldg(row + c0), t1 = __ldg(row + c1);
                        const float2 v = make_float2(fmaf(ub.x, t0.y, t0.x),
                                                     fmaf(ub.y, t1.y, t1.x));
                        acc[i][r >> 1] = __ffma2_rn(v, w, acc[i][r >> 1]);
                    }
                }
            }
        }
    }
    if (__syncthreads_or(gave_up) && tid == 0) {
        atomicAdd(&g_wait_timeouts, 1ull);
        if (gave_up) mbar_wait(bar, phase, kWaitTries);
    }
    if (x >= half) return;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int y = y0 + 8 * r;
        if (y >= half) continue;
        // pixel R^k P for row i: k = i (DIR +1) or -i mod 4 (DIR -1)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float v = (r & 1) ? acc[i][r >> 1].y : acc[i][r >> 1].x;
            const int k = dir > 0 ? i : (4 - i) & 3;
            int px = x, py = y;
            if (k == 1) px = y, py = W - 1 - x;
            else if (k == 2) px = W - 1 - x, py = W - 1 - y;
            else if (k == 3) px = W - 1 - y, py = x;
            vol[(size_t)py * W + px] += v * inv;
        }
    }
}

// 4 pixels per thread (32 x 32-pixel tiles of the first quadrant), 16 views
// per pass (64 rows of 82 pairs, 43 KB): measured fastest of the shapes
// tried (2 or 4 pixels, 8 or 16 views, windows of 64, 80 or 128 pairs), at
// n = 1536 / 2048 / 4096 14-16 % below the per-view kernel.
template <int MINB>
__global__ void __launch_bounds__(256, MINB)
    k_bwd2d_sym(float *__restrict__ vol, const float2 *__restrict__ S,
                const float4 *__restrict__ proj, int W, int det, int nangles, float sx, float ox,
                float ds, int dir) {
    bwd2d_sym_tile<kSymR, kSymNV, kSymWin>(vol, S, proj, W, det, nangles, sx, ox, ds, dir,
                                           blockIdx.x, blockIdx.y);
}

// MINB: resident blocks per SM the register allocation must allow
template <int MINB, bool PK, bool MAGIC = false, int VU = 2, bool CPA = false, bool ABS = false,
          bool MAPQ = false, bool BULK = false, int R = kSmRows>
__global__ void __launch_bounds__(256, MINB)
    k_bwd2d_smem(float *__restrict__ vol, const float2 *__restrict__ S,
                 const float4 *__restrict__ proj, int W, int H, int det, int nangles, float sx,
                 float sy, float ox, float oy, float ds) {
    bwd2d_smem_tile<PK, MAGIC, VU, CPA, ABS, MAPQ, BULK, R>(vol, S, proj, W, H, det, nangles,
                                                            sx, sy, ox, oy, ds, blockIdx.x,
                                                            blockIdx.y);
}

}  // namespace

namespace {

// ------------------------------------------------------------ batches

// A batch runs every stage of many 2D problems (any sizes, geometries) as
// one launch over a work list: stage s of problem i owns the blocks
// [start[s][i], start[s][i + 1]) of the launch, and each block finds its
// problem by binary search over those starts (batch_problem), then runs the
// single-problem tile or ray code on it.

__global__ void __launch_bounds__(256)
    k_batch_relayout2d(const Prob2d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.W + 2 * kPad + kTile - 1) / kTile;
    relayout2d_tile(q.vol, q.W, q.H, q.layA, q.layB, q.pa, q.pb, local % gx, local / gx);
}

__global__ void __launch_bounds__(256)
    k_batch_relayout2d_abs(const Prob2d *__restrict__ probs, const int *__restrict__ start,
                           int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.W + 2 * kPad + kTile - 1) / kTile;
    relayout2d_tile<true>(q.vol, q.W, q.H, q.layA, q.layB, q.pa, q.pb, local % gx, local / gx);
}

// The chunked forward's default shape (484) over a work list: each block one
// bundle of one problem, the same code and shared memory as the single launch.
__global__ void __launch_bounds__(256, 3)
    k_batch_fwd2d_cslab(const Prob2d *__restrict__ probs, const int *__restrict__ start,
                        int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.det + 127) / 128, gy = (q.nangles + 7) / 8;
    cslab_bundle<16, 256, 128, true, false, 2, 8, 3, 2, true, true>(
        q.layA, q.layB, q.sino, q.src, q.u0, q.du, q.W, q.H, q.det, q.nangles, q.sx, q.sy, q.pa,
        q.pb, local % gx, (local / gx) % gy, local / (gx * gy));
}

__global__ void __launch_bounds__(256)
    k_batch_fwd2d(const Prob2d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.det + 31) / 32;
    fwd2d_ray(q.layA, q.layB, q.sino, q.src, q.u0, q.du, q.W, q.H, q.det, q.nangles, q.sx, q.sy,
              q.pa, q.pb, (local % gx) * 32 + threadIdx.x, (local / gx) * 8 + threadIdx.y);
}

__global__ void __launch_bounds__(256)
    k_batch_relayout_sino2d(const Prob2d *__restrict__ probs, const int *__restrict__ start,
                            int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const long long idx = (long long)(blockIdx.x - start[i]) * blockDim.x + threadIdx.x;
    relayout_sino2d_elem<true>(q.sino, q.det, q.nangles, q.sinoP, idx);
}

// The staged tile of the single-problem default (packed rows, round-down
// floor, window rows by bulk copies, view loop unrolled 4 times,
// absolute-position pairs, 8 x 4-pixel warps), so results equal it bit for
// bit.
__global__ void __launch_bounds__(256, 4)
    k_batch_bwd2d(const Prob2d *__restrict__ probs, const int *__restrict__ start, int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.W + 31) / 32;
    bwd2d_smem_tile<true, true, 4, true, true, true, true>(q.vol, q.sinoP, q.bproj, q.W, q.H,
                                                           q.det, q.nangles, q.sx, q.sy, q.ox,
                                                           q.oy, q.ds, local % gx, local / gx);
}

// The quarter-turn symmetric tile of the single-problem default for the
// problems whose plan has the symmetry (their first quadrant's tiles).
__global__ void __launch_bounds__(256, 4)
    k_batch_bwd2d_sym(const Prob2d *__restrict__ probs, const int *__restrict__ start,
                      int count) {
    const int i = batch_problem(start, count, blockIdx.x);
    const Prob2d &q = probs[i];
    const int local = blockIdx.x - start[i];
    const int gx = (q.W / 2 + 31) / 32;
    bwd2d_sym_tile<kSymR, kSymNV, kSymWin>(q.vol, q.sinoP, q.bproj, q.W, q.det, q.nangles, q.sx,
                                           q.ox, q.ds, q.bwd_sym, local % gx, local / gx);
}

}  // namespace

// Blocks of each batched stage for one problem (the launch shapes of the
// single-problem kernels above).
void batch_blocks(const Plan2d &p, int blocks[kBatchStages]) {
    blocks[0] = ceil_div(p.W + 2 * kPad, kTile) * ceil_div(p.H + 2 * kPad, kTile);
    blocks[1] = ceil_div(p.det, 32) * ceil_div(p.nangles, 8);
    blocks[2] = (int)ceil_div((long long)p.pitchS() * p.nangles, 256);
    blocks[3] = p.bwd_sym ? 0 : ceil_div(p.W, 32) * ceil_div(p.H, 8 * kSmRows);
    blocks[10] = p.bwd_sym ? ceil_div(p.W / 2, 32) * ceil_div(p.W / 2, 8 * kSymR) : 0;
    // matched adjoint: 1024 float4 zeroed per block, one ray per thread in
    // 32 x 8 blocks, one voxel per thread in 32 x 8 blocks
    blocks[4] = (int)ceil_div((long long)(adj2d_quad_elems(p, true) + adj2d_quad_elems(p, false)),
                              1024);
    blocks[5] = ceil_div(p.det, 32) * ceil_div(p.nangles, 8);
    blocks[6] = ceil_div(p.W, 32) * ceil_div(p.H, 8);
    // "plans" forward: the chunked bundles (with their re-layout) where the
    // plan's own forward is the chunked shape compiled for batches, else the
    // texture rays
    const bool chunked = batch_chunked(p);
    blocks[7] = chunked ? blocks[0] : 0;
    blocks[8] = chunked ? ceil_div(p.det, 128) * ceil_div(p.nangles, 8) * 2 : 0;
    blocks[9] = chunked ? 0 : blocks[1];
}

bool batch_chunked(const Plan2d &p) {
    return p.algo_fwd == 4 && p.fwd_chunk_rows == kBatchChunkShape &&
           std::max(p.pitchA(), p.pitchB()) < 32768;
}

int launch_batch2d_fwd_plans(const Prob2d *d_probs, const std::vector<Prob2d> &probs,
                             int active, const int *starts, const int totals[kBatchStages],
                             int count, cudaStream_t s) {
    int rc = launch_batch2d_fwd_tex_stage(d_probs, probs, active, starts + 9 * (count + 1),
                                          totals[9], true, s);
    if (rc) return rc;
    if (totals[8] == 0) return CG_OK;
    k_batch_relayout2d_abs<<<totals[7], dim3(32, 8), 0, s>>>(d_probs, starts + 7 * (count + 1),
                                                             count);
    CG_TRY_CUDA(cudaGetLastError());
    constexpr int smem = 2 * (int)sizeof(float2) * (16 + 1) * 256;
    if ((rc = ensure_smem_attr((const void *)k_batch_fwd2d_cslab, smem))) return rc;
    k_batch_fwd2d_cslab<<<totals[8], 256, smem, s>>>(d_probs, starts + 8 * (count + 1), count);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_batch2d(const Prob2d *probs, const int *starts, const int totals[kBatchStages],
                   int count, bool forward, cudaStream_t s) {
    const dim3 tile(32, 8);
    if (forward) {
        k_batch_relayout2d<<<totals[0], tile, 0, s>>>(probs, starts, count);
        CG_TRY_CUDA(cudaGetLastError());
        k_batch_fwd2d<<<totals[1], tile, 0, s>>>(probs, starts + (count + 1), count);
    } else {
        k_batch_relayout_sino2d<<<totals[2], 256, 0, s>>>(probs, starts + 2 * (count + 1), count);
        CG_TRY_CUDA(cudaGetLastError());
        if (totals[3] > 0)
            k_batch_bwd2d<<<totals[3], tile, 0, s>>>(probs, starts + 3 * (count + 1), count);
        CG_TRY_CUDA(cudaGetLastError());
        if (totals[10] > 0)
            k_batch_bwd2d_sym<<<totals[10], tile, 0, s>>>(probs, starts + 10 * (count + 1),
                                                          count);
    }
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

// ------------------------------------------------------------ launchers

int launch_plan2d_tables(Plan2d &p, cudaStream_t s) {
    const float det_ext = (float)p.det * p.ds;
    const float extx = (float)p.W * p.sx, exty = (float)p.H * p.sy;
    k_plan2d_tables<<<ceil_div(p.nangles, 128), 128, 0, s>>>(
        p.nangles, p.d_angles, p.d_DSO, p.d_DSD, det_ext, p.ds, p.doff, p.sx, p.sy, p.ox, p.oy,
        extx, exty, p.d_src, p.d_u0, p.d_du, p.d_bmeta, p.d_bproj);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_relayout2d(const Plan2d &p, const float *vol, cudaStream_t s) {
    dim3 grid(ceil_div(p.W + 2 * kPad, kTile), ceil_div(p.H + 2 * kPad, kTile));
    // the chunked forward's absolute-position shapes read the ABS form
    const bool abs_form = (p.algo_fwd == 4 || p.algo_fwd == 5) && cslab_abs(p.fwd_chunk_rows);
    auto kernel = abs_form ? k_relayout2d<true> : k_relayout2d<false>;
    kernel<<<grid, dim3(32, 8), 0, s>>>(vol, p.W, p.H, p.d_layA, p.d_layB, p.pitchA(),
                                        p.pitchB());
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_forward2d(const Plan2d &p, float *sino, cudaStream_t s) {
    dim3 block(p.fwd_bx, p.fwd_by);
    dim3 grid(ceil_div(p.det, p.fwd_bx), ceil_div(p.nangles, p.fwd_by));
    if (grid.y > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    k_fwd2d<<<grid, block, 0, s>>>(p.d_layA, p.d_layB, sino, p.d_src, p.d_u0, p.d_du, p.W, p.H,
                                   p.det, p.nangles, p.sx, p.sy, p.pitchA(), p.pitchB());
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_relayout_sino2d(const Plan2d &p, const float *sino, cudaStream_t s) {
    const long long n = (long long)p.pitchS() * p.nangles;
    // the staged backprojector's absolute-position shapes read the ABS form
    const bool abs_form = (p.algo_bwd == 2 || p.algo_bwd == 3) && bwd_abs(p.bwd_min_blocks);
    auto kernel = abs_form ? k_relayout_sino2d<true> : k_relayout_sino2d<false>;
    kernel<<<ceil_div(n, 256), 256, 0, s>>>(sino, p.det, p.nangles, p.d_sinoP);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

// Streaming multiprocessors of the current device (looked up once per device).
int sm_count() {
    static int counts[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!counts[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 152;
        counts[dev] = n;
    }
    return counts[dev];
}

int sym_quadrant_blocks(int W) { return ceil_div(W / 2, 32) * ceil_div(W / 2, 8 * kSymR); }

int launch_backward2d_smem(const Plan2d &p, float *vol, cudaStream_t s) {
    if (p.bwd_sym != 0) {
        // the first quadrant's tiles, each with its three turned copies
        const int half = p.W / 2;
        const dim3 grid(ceil_div(half, 32), ceil_div(half, 8 * kSymR));
        k_bwd2d_sym<4><<<grid, dim3(32, 8), 0, s>>>(vol, p.d_sinoP, p.d_bproj, p.W, p.det,
                                                 p.nangles, p.sx, p.ox, p.ds, p.bwd_sym);
        CG_TRY_CUDA(cudaGetLastError());
        return CG_OK;
    }
    // tiles of 32 x 64 pixels; an image whose tiles would not give every SM
    // two blocks takes 32 x 16-pixel tiles (two pixels per thread) instead,
    // four times the blocks, the same sums
    const bool small = (long long)ceil_div(p.W, 32) * ceil_div(p.H, 8 * kSmRows) < 2LL * sm_count();
    const dim3 grid(ceil_div(p.W, 32), ceil_div(p.H, 8 * (small ? 2 : kSmRows)));
    auto go = [&](auto kernel) {
        kernel<<<grid, dim3(32, 8), 0, s>>>(vol, p.d_sinoP, p.d_bproj, p.W, p.H, p.det,
                                            p.nangles, p.sx, p.sy, p.ox, p.oy, p.ds);
    };
    // the default (68) and the autotuner's other candidates (48: the same
    // staged pair by pair with cp.async; 27: (t, d) pairs, 32 x 1-pixel warps,
    // view loop unrolled twice)
    switch (p.bwd_min_blocks) {
        case 27:
            small ? go(k_bwd2d_smem<4, true, true, 2, true, false, false, false, 2>)
                  : go(k_bwd2d_smem<4, true, true, 2, true>);
            break;
        case 48:
            small ? go(k_bwd2d_smem<4, true, true, 4, true, true, true, false, 2>)
                  : go(k_bwd2d_smem<4, true, true, 4, true, true, true>);
            break;
        default:
            small ? go(k_bwd2d_smem<4, true, true, 4, true, true, true, true, 2>)
                  : go(k_bwd2d_smem<4, true, true, 4, true, true, true, true>);
            break;
    }
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_backward2d(const Plan2d &p, float *vol, cudaStream_t s) {
    dim3 grid(ceil_div(p.W, 32), ceil_div(p.H, 32));
    k_bwd2d<<<grid, dim3(32, 8), 0, s>>>(vol, p.d_sinoP, p.d_bmeta, p.W, p.H, p.det, p.nangles,
                                         p.sx, p.sy, p.ox, p.oy, p.ds);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
