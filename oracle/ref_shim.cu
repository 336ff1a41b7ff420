// ref_shim.cu -- C-ABI wrapper over the reference's own CUDA operators.
//
// TEST INFRASTRUCTURE ONLY: it lets the tests and the golden-vector script
// run the UNMODIFIED reference kernels (curadon's header-only library,
// include/curadon/...) on the same inputs as ours.  It is compiled by
// oracle/build_ref.py into oracle/_ref/ and never linked into the product.
//
// Each function repeats the marshaling the reference's nanobind extension
// does before it calls the library (python/standalone/src/):
//   ref_plan2d_create  <- plan.cu:34-56   (axis swap, thrust vectors)
//   ref_forward2d      <- forward.cu:77-90 (spans {W,H}, {det, nangles})
//   ref_backward2d     <- backward.cu:75-87
//   ref_forward2d_t / ref_backward2d_t  <- the f16 instantiations of both
//   ref_forward3d      <- forward.cu:23-75 (axis swaps, psi/phi naming swap)
//   ref_backward3d     <- backward.cu:20-72
#include <cstdint>
#include <vector>

#include <thrust/device_vector.h>

#include "curadon/backward.hpp"
#include "curadon/detail/plan/plan_2d.hpp"
#include "curadon/forward.hpp"
#include "curadon/image.hpp"
#include "curadon/measurement.hpp"

// The typed instantiations of forward.cu:77-90 / backward.cu:75-87: T is the
// volume's element type, U the sinogram's (float or __half).
template <class T, class U>
static void fwd2d_typed(curad::plan_2d &p, void *vol, void *sino) {
    curad::device_span_2d<T> vol_span(p.device_id(), (T *)vol, p.vol_shape());
    curad::device_span_2d<U> sino_span(p.device_id(), (U *)sino, {p.det_count(), p.nangles()});
    curad::fp::forward_2d<T, U>(vol_span, sino_span, p);
}

template <class T, class U>
static void bwd2d_typed(curad::plan_2d &p, void *vol, void *sino) {
    curad::device_span_2d<T> vol_span(p.device_id(), (T *)vol, p.vol_shape());
    curad::device_span_2d<U> sino_span(p.device_id(), (U *)sino, {p.det_count(), p.nangles()});
    curad::bp::backproject_2d(vol_span, sino_span, p);
}

extern "C" {

static curad::precision prec_of(uint32_t bits) {
    return bits == 16 ? curad::precision::HALF : curad::precision::SINGLE;
}

void *ref_plan2d_create(uint64_t device, const uint64_t py_vol_shape[2],
                        const float py_vol_spacing[2], const float py_vol_offset[2],
                        uint64_t det_count, float det_spacing, float det_offset, const float *DSO,
                        const float *DSD, const float *angles, uint64_t n, float det_pitch,
                        float COR, uint32_t vol_prec, uint32_t det_prec) {
    thrust::device_vector<float> gpu_angles(angles, angles + n);
    thrust::device_vector<float> gpu_dso(DSO, DSO + n);
    thrust::device_vector<float> gpu_dsd(DSD, DSD + n);
    curad::vec2u vol_shape{py_vol_shape[1], py_vol_shape[0]};
    curad::vec2f vol_spacing{py_vol_spacing[1], py_vol_spacing[0]};
    curad::vec2f vol_offset{py_vol_offset[1], py_vol_offset[0]};
    return new curad::plan_2d(device, prec_of(vol_prec), vol_shape, vol_spacing, vol_offset,
                              prec_of(det_prec), det_count, det_spacing, det_offset, gpu_dso,
                              gpu_dsd, gpu_angles, det_pitch, COR);
}

void ref_plan2d_destroy(void *plan) { delete static_cast<curad::plan_2d *>(plan); }

void ref_plan2d_tables(void *plan, float *src, float *u0, float *du) {
    auto &p = *static_cast<curad::plan_2d *>(plan);
    const size_t bytes = sizeof(curad::vec2f) * p.nangles();
    cudaMemcpy(src, p.sources().data(), bytes, cudaMemcpyDeviceToHost);
    cudaMemcpy(u0, p.u_origins().data(), bytes, cudaMemcpyDeviceToHost);
    cudaMemcpy(du, p.delta_us().data(), bytes, cudaMemcpyDeviceToHost);
}

void ref_forward2d(void *plan, float *vol, float *sino) {
    auto &p = *static_cast<curad::plan_2d *>(plan);
    curad::device_span_2d<float> vol_span(p.device_id(), vol, p.vol_shape());
    curad::device_span_2d<float> sino_span(p.device_id(), sino, {p.det_count(), p.nangles()});
    curad::fp::forward_2d<float, float>(vol_span, sino_span, p);
}

void ref_backward2d(void *plan, float *vol, float *sino) {
    auto &p = *static_cast<curad::plan_2d *>(plan);
    curad::device_span_2d<float> vol_span(p.device_id(), vol, p.vol_shape());
    curad::device_span_2d<float> sino_span(p.device_id(), sino, {p.det_count(), p.nangles()});
    curad::bp::backproject_2d(vol_span, sino_span, p);
}

void ref_forward2d_t(void *plan, void *vol, void *sino, int vol_bits, int sino_bits) {
    auto &p = *static_cast<curad::plan_2d *>(plan);
    using curad::f16;
    if (vol_bits == 16)
        sino_bits == 16 ? fwd2d_typed<f16, f16>(p, vol, sino) : fwd2d_typed<f16, float>(p, vol, sino);
    else
        sino_bits == 16 ? fwd2d_typed<float, f16>(p, vol, sino) : fwd2d_typed<float, float>(p, vol, sino);
}

void ref_backward2d_t(void *plan, void *vol, void *sino, int vol_bits, int sino_bits) {
    auto &p = *static_cast<curad::plan_2d *>(plan);
    using curad::f16;
    if (vol_bits == 16)
        sino_bits == 16 ? bwd2d_typed<f16, f16>(p, vol, sino) : bwd2d_typed<f16, float>(p, vol, sino);
    else
        sino_bits == 16 ? bwd2d_typed<float, f16>(p, vol, sino) : bwd2d_typed<float, float>(p, vol, sino);
}

static curad::device_measurement<float>
make_measurement(float *sino, const uint64_t det_shape[2], const float det_spacing[2],
                 const float det_offset[2], const float det_rotation[3], const float *a0,
                 const float *a1, const float *a2, uint64_t n, float DSO, float DSD, float COR) {
    curad::vec3u curad_det_shape{det_shape[1], det_shape[0], n};
    curad::vec2f curad_det_spacing{det_spacing[1], det_spacing[0]};
    curad::vec2f curad_det_offset{det_offset[1], det_offset[0]};
    // The extension receives geom.angles[0], [1], [2] positionally and hands
    // them to set_angles(phi, theta, psi) in that order.
    std::vector<float> cpu_psi(a0, a0 + n);
    std::vector<float> cpu_theta(a1, a1 + n);
    std::vector<float> cpu_phi(a2, a2 + n);
    curad::device_measurement<float> m(0, sino, curad_det_shape, curad_det_spacing,
                                       curad_det_offset);
    m.set_angles(cpu_psi, cpu_theta, cpu_phi);
    m.set_distance_source_to_detector(DSD);
    m.set_distance_source_to_object(DSO);
    m.set_center_of_rotation_correction(COR);
    m.set_pitch(det_rotation[0]);
    m.set_roll(det_rotation[1]);
    m.set_yaw(det_rotation[2]);
    return m;
}

void ref_forward3d(float *vol, const uint64_t vol_shape[3], const float vol_spacing[3],
                   const float vol_offset[3], float *sino, const float *a0, const float *a1,
                   const float *a2, uint64_t n, const uint64_t det_shape[2],
                   const float det_spacing[2], const float det_offset[2],
                   const float det_rotation[3], float DSO, float DSD, float COR) {
    curad::vec3u s{vol_shape[2], vol_shape[1], vol_shape[0]};
    curad::vec3f sp{vol_spacing[2], vol_spacing[1], vol_spacing[0]};
    curad::vec3f off{vol_offset[2], vol_offset[1], vol_offset[0]};
    curad::device_volume<float> v(0, vol, s, sp, off);
    auto m = make_measurement(sino, det_shape, det_spacing, det_offset, det_rotation, a0, a1, a2,
                              n, DSO, DSD, COR);
    curad::fp::forward_3d(v, m);
}

void ref_backward3d(float *vol, const uint64_t vol_shape[3], const float vol_spacing[3],
                    const float vol_offset[3], float *sino, const float *a0, const float *a1,
                    const float *a2, uint64_t n, const uint64_t det_shape[2],
                    const float det_spacing[2], const float det_offset[2],
                    const float det_rotation[3], float DSO, float DSD, float COR) {
    curad::vec3u s{vol_shape[2], vol_shape[1], vol_shape[0]};
    curad::vec3f sp{vol_spacing[2], vol_spacing[1], vol_spacing[0]};
    curad::vec3f off{vol_offset[2], vol_offset[1], vol_offset[0]};
    curad::device_volume<float> v(0, vol, s, sp, off);
    auto m = make_measurement(sino, det_shape, det_spacing, det_offset, det_rotation, a0, a1, a2,
                              n, DSO, DSD, COR);
    curad::bp::backproject_3d(v, m);
}

int ref_sync(void) { return (int)cudaDeviceSynchronize(); }

}  // extern "C"
