// Small runtime helpers and FP16 storage for the 2D operators (the reference's f16 paths,
// python/standalone/src/forward.cu:107-135 and backward.cu:104-135).
//
// Values are stored as IEEE half and computed in FP32: a half volume or
// sinogram is widened into a plan scratch buffer before the FP32 kernels run
// (the texture unit of the reference widens half texels the same way), a
// half sinogram is written by rounding each FP32 ray sum to nearest (the
// reference's float -> __half assignment), and a half volume receives the
// backprojection as half(acc / ds) added in half arithmetic, as the
// reference's `volume[i] += accum * inv_u_spacing` does for T = __half.
#include <cuda_fp16.h>

#include <map>
#include <mutex>

#include "common.cuh"

namespace cg {
namespace {

__global__ void k_half_to_float(const __half *__restrict__ in, float *__restrict__ out,
                                long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = __half2float(in[i]);
}

__global__ void k_float_to_half(const float *__restrict__ in, __half *__restrict__ out,
                                long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(in[i]);
}

__global__ void k_add_to_half(__half *__restrict__ vol, const float *__restrict__ add,
                              long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        vol[i] = __hadd(vol[i], __float2half_rn(add[i]));
}

dim3 grid_for(long long n) { return dim3((unsigned)std::min<long long>(ceil_div(n, 256), 152 * 16)); }

}  // namespace

int ensure_smem_attr(const void *func, int bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> done;
    int dev = 0;
    CG_TRY_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    int &have = done[{dev, func}];
    if (have < bytes) {
        CG_TRY_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        have = bytes;
    }
    return CG_OK;
}

int ensure_half_scratch(Plan2d &p, bool vol, bool sino) {
    if (vol && !p.d_vol32)
        CG_TRY_CUDA(cudaMalloc(&p.d_vol32, sizeof(float) * (size_t)p.W * p.H));
    if (sino && !p.d_sino32)
        CG_TRY_CUDA(cudaMalloc(&p.d_sino32, sizeof(float) * (size_t)p.det * p.nangles));
    return CG_OK;
}

int widen_half(const void *in, float *out, long long n, cudaStream_t s) {
    k_half_to_float<<<grid_for(n), 256, 0, s>>>(static_cast<const __half *>(in), out, n);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int narrow_to_half(const float *in, void *out, long long n, cudaStream_t s) {
    k_float_to_half<<<grid_for(n), 256, 0, s>>>(in, static_cast<__half *>(out), n);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int add_into_half(void *vol, const float *add, long long n, cudaStream_t s) {
    k_add_to_half<<<grid_for(n), 256, 0, s>>>(static_cast<__half *>(vol), add, n);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
