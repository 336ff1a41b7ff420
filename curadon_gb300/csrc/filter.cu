// filter.cu -- row filtering for filtered backprojection (FBP).
//
// The reference's FBP (examples/fbp.py:27-56) multiplies each sinogram row's
// length-N DFT by a real frequency response w (|linspace(-1,1,N)|, optionally
// apodised), fftshifted, and keeps the real part of the inverse DFT.  For a
// real row that is exactly the circular convolution of the row with
// h = Re(IDFT(fftshift(w))).  This kernel evaluates that convolution
// directly, out[r][k] = scale * sum_j pre[j] in[r][j] h[(k - j) mod N], with
// the optional per-cell pre-weight (e.g. fan-beam cosine weighting) fused in.
//
// CURADON_GB300_FILTER=scalar selects the one-row kernel everywhere (the
// packed one computes the same bits; see k_filter_rows_pk).
//
// Block = 256 threads x 4 consecutive outputs each = 1024 outputs of RB rows;
// the RB input rows and h live in shared memory; as j advances, the four h
// values a thread needs shift by one, so each step loads one new h value and
// RB row values (broadcast) for 4 * RB fused multiply-adds.
#include "common.cuh"

namespace cg {
namespace {

constexpr int kFiltThreads = 256;
constexpr int kFiltOut = 4;  // outputs per thread

template <int RB>
__global__ void __launch_bounds__(kFiltThreads)
    k_filter_rows(const float *__restrict__ in, float *__restrict__ out,
                  const float *__restrict__ h, const float *__restrict__ pre, int nrows, int N,
                  float scale) {
    extern __shared__ float smem[];
    float *sh = smem;            // N
    float *srow = smem + N;      // RB x N
    const int r0 = blockIdx.y * RB;
    for (int i = threadIdx.x; i < N; i += kFiltThreads) sh[i] = h[i];
    for (int r = 0; r < RB; ++r) {
        const bool ok = r0 + r < nrows;
        const float *row = in + (size_t)(r0 + r) * N;
        for (int i = threadIdx.x; i < N; i += kFiltThreads)
            srow[r * N + i] = ok ? (pre ? row[i] * pre[i] : row[i]) : 0.f;
    }
    __syncthreads();
    const int k0 = (blockIdx.x * kFiltThreads + threadIdx.x) * kFiltOut;
    if (k0 >= N) return;
    float acc[RB][kFiltOut];
#pragma unroll
    for (int r = 0; r < RB; ++r)
#pragma unroll
        for (int i = 0; i < kFiltOut; ++i) acc[r][i] = 0.f;
    // hw[i] = h[(k0 + i - j) mod N] for the current j (indices clamped to the
    // row for outputs past its end, which are not stored)
    float hw[kFiltOut];
#pragma unroll
    for (int i = 0; i < kFiltOut; ++i) hw[i] = sh[(k0 + i) % N];
    int hidx = k0;  // (k0 - j) mod N
    for (int j = 0; j < N; ++j) {
#pragma unroll
        for (int r = 0; r < RB; ++r) {
            const float s = srow[r * N + j];
#pragma unroll
            for (int i = 0; i < kFiltOut; ++i) acc[r][i] = fmaf(s, hw[i], acc[r][i]);
        }
        // advance to j + 1: shift the window, load h[(k0 - j - 1) mod N]
        hidx = hidx == 0 ? N - 1 : hidx - 1;
#pragma unroll
        for (int i = kFiltOut - 1; i > 0; --i) hw[i] = hw[i - 1];
        hw[0] = sh[hidx];
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
        if (r0 + r >= nrows) break;
        float *o = out + (size_t)(r0 + r) * N;
#pragma unroll
        for (int i = 0; i < kFiltOut; ++i)
            if (k0 + i < N) o[k0 + i] = acc[r][i] * scale;
    }
}

// The same convolution on pairs of rows: the rows 2p and 2p + 1 of the block
// are interleaved in shared memory and h is stored duplicated, so one packed
// FP32 FMA (`__ffma2_rn`) advances one output of two rows; the accumulation
// order of every output is that of k_filter_rows.
template <int RB>
__global__ void __launch_bounds__(kFiltThreads)
    k_filter_rows_pk(const float *__restrict__ in, float *__restrict__ out,
                     const float *__restrict__ h, const float *__restrict__ pre, int nrows, int N,
                     float scale) {
    static_assert(RB % 2 == 0, "row pairs");
    extern __shared__ float2 smem2[];
    float2 *sh = smem2;         // N: (h, h)
    float2 *srow = smem2 + N;   // RB / 2 x N: (row 2p, row 2p + 1)
    const int r0 = blockIdx.y * RB;
    for (int i = threadIdx.x; i < N; i += kFiltThreads) sh[i] = make_float2(h[i], h[i]);
    for (int rp = 0; rp < RB / 2; ++rp) {
        const int ra = r0 + 2 * rp, rb = ra + 1;
        const float *rowa = in + (size_t)ra * N, *rowb = in + (size_t)rb * N;
        for (int i = threadIdx.x; i < N; i += kFiltThreads) {
            const float w = pre ? pre[i] : 1.f;
            srow[rp * N + i] = make_float2(ra < nrows ? rowa[i] * w : 0.f,
                                           rb < nrows ? rowb[i] * w : 0.f);
        }
    }
    __syncthreads();
    const int k0 = (blockIdx.x * kFiltThreads + threadIdx.x) * kFiltOut;
    if (k0 >= N) return;
    float2 acc[RB / 2][kFiltOut];
#pragma unroll
    for (int rp = 0; rp < RB / 2; ++rp)
#pragma unroll
        for (int i = 0; i < kFiltOut; ++i) acc[rp][i] = make_float2(0.f, 0.f);
    float2 hw[kFiltOut];
#pragma unroll
    for (int i = 0; i < kFiltOut; ++i) hw[i] = sh[(k0 + i) % N];
    int hidx = k0;
#pragma unroll 4
    for (int j = 0; j < N; ++j) {
#pragma unroll
        for (int rp = 0; rp < RB / 2; ++rp) {
            const float2 sv = srow[rp * N + j];
#pragma unroll
            for (int i = 0; i < kFiltOut; ++i) acc[rp][i] = __ffma2_rn(sv, hw[i], acc[rp][i]);
        }
        hidx = hidx == 0 ? N - 1 : hidx - 1;
#pragma unroll
        for (int i = kFiltOut - 1; i > 0; --i) hw[i] = hw[i - 1];
        hw[0] = sh[hidx];
    }
#pragma unroll
    for (int rp = 0; rp < RB / 2; ++rp) {
        const int ra = r0 + 2 * rp;
#pragma unroll
        for (int i = 0; i < kFiltOut; ++i) {
            if (k0 + i >= N) continue;
            if (ra < nrows) out[(size_t)ra * N + k0 + i] = acc[rp][i].x * scale;
            if (ra + 1 < nrows) out[(size_t)(ra + 1) * N + k0 + i] = acc[rp][i].y * scale;
        }
    }
}

template <int RB>
int launch_rb_pk(const float *in, float *out, const float *h, const float *pre, int nrows, int N,
                 float scale, cudaStream_t s) {
    const size_t smem = sizeof(float2) * (size_t)N * (RB / 2 + 1);
    if (int rc = ensure_smem_attr((const void *)k_filter_rows_pk<RB>, (int)smem)) return rc;
    dim3 grid(ceil_div(N, kFiltThreads * kFiltOut), ceil_div(nrows, RB));
    k_filter_rows_pk<RB><<<grid, kFiltThreads, smem, s>>>(in, out, h, pre, nrows, N, scale);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

template <int RB>
int launch_rb(const float *in, float *out, const float *h, const float *pre, int nrows, int N,
              float scale, cudaStream_t s) {
    const size_t smem = sizeof(float) * (size_t)N * (RB + 1);
    if (int rc = ensure_smem_attr((const void *)k_filter_rows<RB>, (int)smem)) return rc;
    dim3 grid(ceil_div(N, kFiltThreads * kFiltOut), ceil_div(nrows, RB));
    k_filter_rows<RB><<<grid, kFiltThreads, smem, s>>>(in, out, h, pre, nrows, N, scale);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

}  // namespace

int launch_filter_rows(const float *in, float *out, const float *h, const float *pre, int nrows,
                       int N, float scale, cudaStream_t s) {
    constexpr size_t kMaxSmem = 227 * 1024;
    static const bool packed = [] {
        const char *v = getenv("CURADON_GB300_FILTER");
        return !(v && std::string(v) == "scalar");
    }();
    // packed row pairs while two blocks of them fit an SM (measured: -11 % at
    // 1449 cells, -8 % at 725; at 2897 cells only one block fits, +6 %)
    if (packed && 2 * (sizeof(float) * (size_t)N * 10 + 1024) <= 228 * 1024)
        return launch_rb_pk<8>(in, out, h, pre, nrows, N, scale, s);
    if (sizeof(float) * (size_t)N * 9 <= kMaxSmem)
        return launch_rb<8>(in, out, h, pre, nrows, N, scale, s);
    if (sizeof(float) * (size_t)N * 5 <= kMaxSmem)
        return launch_rb<4>(in, out, h, pre, nrows, N, scale, s);
    if (sizeof(float) * (size_t)N * 2 <= kMaxSmem)
        return launch_rb<1>(in, out, h, pre, nrows, N, scale, s);
    return set_error(CG_ERR_INVALID, "row too long for the shared-memory filter (max 29056)");
}

}  // namespace cg
