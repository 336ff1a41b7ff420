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
    if (sizeof(float) * (size_t)N * 9 <= kMaxSmem)
        return launch_rb<8>(in, out, h, pre, nrows, N, scale, s);
    if (sizeof(float) * (size_t)N * 5 <= kMaxSmem)
        return launch_rb<4>(in, out, h, pre, nrows, N, scale, s);
    if (sizeof(float) * (size_t)N * 2 <= kMaxSmem)
        return launch_rb<1>(in, out, h, pre, nrows, N, scale, s);
    return set_error(CG_ERR_INVALID, "row too long for the shared-memory filter (max 29056)");
}

}  // namespace cg
