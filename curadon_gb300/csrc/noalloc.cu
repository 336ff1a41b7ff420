// noalloc.cu -- a 2D backprojection entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: a serving process whose device memory
// is reserved up front by its own pool allocator, a real-time reconstruction
// loop that must not stall on the allocator or fail on fragmentation, or a
// plugin host that forbids allocations by the libraries it loads.  For them,
// cg_backward_2d_static runs the same backprojection as cg_plan2d_create +
// cg_backward_2d, but every byte of scratch it needs -- the staged per-view
// geometry, the per-view tables and the pair-packed, zero-padded copy of the
// sinogram -- lives in one file-scope device array of fixed size
// (kStaticScratchBytes) that the module reserves when the library is loaded;
// every GPU that loads the library holds it until the process exits.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it (a host
// variable naming the array is only a host-side stand-in, not a device
// address).  That first call should therefore come before any stream capture.
//
// Sharing: all calls share the one array and it keeps the last call's
// contents.  Each call overwrites everything it reads (the tables and the
// whole padded sinogram copy, padding included), so nothing has to start at
// zero; but two calls that overlap on the GPU -- on different streams, or
// from different threads -- race on the array and must be ordered by the
// caller.
#include <cmath>
#include <string>

#include "common.cuh"

namespace cg {
namespace {

// 16 MiB: e.g. 1024 views x 2000 detector cells.
constexpr size_t kStaticScratchBytes = size_t(16) << 20;
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch in the current context, looked up on
// every call (a lookup allocates nothing, and an address kept from an
// earlier context would be stale after cudaDeviceReset).
int static_scratch(void **out) {
    void *p = nullptr;
    CG_TRY_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
    *out = p;
    return CG_OK;
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" int cg_backward_2d_static(float *volume, const float *sinogram,
                                     const uint64_t vol_shape[2], const float vol_spacing[2],
                                     const float vol_offset[2], uint64_t det_count,
                                     float det_spacing, const float *DSO, const float *DSD,
                                     const float *angles, uint64_t nangles, void *stream) {
    clear_error();
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    CG_REQUIRE(vol_shape && vol_spacing && vol_offset && DSO && DSD && angles,
               "geometry array is NULL");
    CG_REQUIRE(nangles > 0 && nangles <= (1u << 22), "nangles out of range");
    CG_REQUIRE(det_count > 0 && det_count <= (1u << 20), "det_count out of range");
    CG_REQUIRE(vol_shape[0] > 0 && vol_shape[1] > 0 && vol_shape[0] <= (1u << 15) &&
                   vol_shape[1] <= (1u << 15),
               "volume shape out of range");
    CG_REQUIRE(std::isfinite(det_spacing) && det_spacing != 0.f, "det_spacing must be nonzero");

    // scratch layout: staged angles/DSO/DSD, per-view tables, padded sinogram
    const size_t n = nangles;
    const size_t off_ang = 0;
    const size_t off_dso = align256(off_ang + 4 * n);
    const size_t off_dsd = align256(off_dso + 4 * n);
    const size_t off_src = align256(off_dsd + 4 * n);
    const size_t off_u0 = align256(off_src + 8 * n);
    const size_t off_du = align256(off_u0 + 8 * n);
    const size_t off_meta = align256(off_du + 8 * n);
    const size_t off_proj = align256(off_meta + 16 * n);
    const size_t off_sino = align256(off_proj + 32 * n);
    const size_t total = off_sino + 8 * n * (det_count + 2 * kPad);
    if (total > kStaticScratchBytes)
        return set_error(CG_ERR_INVALID,
                         "problem needs " + std::to_string(total) + " bytes of scratch; the "
                         "static scratch holds " + std::to_string(kStaticScratchBytes) +
                         " (a call needs at most 8 x nangles x (det_count + 4) + 84 x nangles "
                         "+ 2040 bytes)");

    void *base = nullptr;
    int rc = static_scratch(&base);
    if (rc) return rc;
    unsigned char *b = static_cast<unsigned char *>(base);

    // A plan that lives on the host stack and points into the static array.
    Plan2d p;
    CG_TRY_CUDA(cudaGetDevice(&p.device));
    p.W = (int)vol_shape[1], p.H = (int)vol_shape[0];
    p.sx = vol_spacing[1], p.sy = vol_spacing[0];
    p.ox = vol_offset[1], p.oy = vol_offset[0];
    p.det = (int)det_count, p.ds = det_spacing, p.doff = 0.f;
    p.nangles = (int)nangles;
    p.d_angles = reinterpret_cast<float *>(b + off_ang);
    p.d_DSO = reinterpret_cast<float *>(b + off_dso);
    p.d_DSD = reinterpret_cast<float *>(b + off_dsd);
    p.d_src = reinterpret_cast<float2 *>(b + off_src);
    p.d_u0 = reinterpret_cast<float2 *>(b + off_u0);
    p.d_du = reinterpret_cast<float2 *>(b + off_du);
    p.d_bmeta = reinterpret_cast<float4 *>(b + off_meta);
    p.d_bproj = reinterpret_cast<float4 *>(b + off_proj);
    p.d_sinoP = reinterpret_cast<float2 *>(b + off_sino);
    apply_algo_env(&p, nullptr);
    // Only the register backprojector (0) and the staged one (2) run on this
    // scratch alone; the texture-unit algorithm would allocate
    // arrays, so an override selecting it falls back to the staged kernel.
    if (p.algo_bwd != 0) p.algo_bwd = 2;

    cudaStream_t s = (cudaStream_t)stream;
    CG_TRY_CUDA(cudaMemcpyAsync(p.d_angles, angles, 4 * n, cudaMemcpyHostToDevice, s));
    CG_TRY_CUDA(cudaMemcpyAsync(p.d_DSO, DSO, 4 * n, cudaMemcpyHostToDevice, s));
    CG_TRY_CUDA(cudaMemcpyAsync(p.d_DSD, DSD, 4 * n, cudaMemcpyHostToDevice, s));
    if ((rc = launch_plan2d_tables(p, s))) return rc;
    if ((rc = launch_relayout_sino2d(p, sinogram, s))) return rc;
    if (p.algo_bwd == 2) return launch_backward2d_smem(p, volume, s);
    return launch_backward2d(p, volume, s);
}
