// capi.cu -- the extern "C" boundary (include/curadon_gb300.h): argument
// checking, plan construction and the operator entry points.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <initializer_list>
#include <utility>
#include <vector>

#include "common.cuh"

namespace cg {

namespace {
thread_local std::string g_last_error;
}

int set_error(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

void clear_error() { g_last_error.clear(); }

template <class T>
static int alloc_copy(T **dst, const T *src, size_t n) {
    CG_TRY_CUDA(cudaMalloc(dst, sizeof(T) * (n ? n : 1)));
    if (n) CG_TRY_CUDA(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    return CG_OK;
}

void free_plan2d(Plan2d *p) {
    if (!p) return;
    if (p->tex_vol) cudaDestroyTextureObject(p->tex_vol);
    if (p->tex_sino) cudaDestroyTextureObject(p->tex_sino);
    if (p->arr_vol) cudaFreeArray(p->arr_vol);
    if (p->arr_sino) cudaFreeArray(p->arr_sino);
    void *ptrs[] = {p->d_angles, p->d_DSO,   p->d_DSD,   p->d_src,   p->d_u0,    p->d_du,
                    p->d_bmeta,  p->d_bproj, p->d_layA,  p->d_layB,  p->d_sinoP, p->d_vol32,
                    p->d_sino32, p->d_quadA, p->d_quadB};
    for (void *q : ptrs)
        if (q) cudaFree(q);
}

void free_plan3d(Plan3d *p) {
    if (!p) return;
    if (p->tex3) cudaDestroyTextureObject(p->tex3);
    if (p->arr3) cudaFreeArray(p->arr3);
    void *ptrs[] = {p->d_forg, p->d_fdu, p->d_fdv, p->d_fsrc, p->d_borg, p->d_bdx,
                    p->d_bdy,  p->d_bdz, p->d_volA, p->d_volB, p->d_sinoP, p->d_quadA,
                    p->d_quadB, p->d_sinoQ, p->d_volQA, p->d_volQB};
    for (void *q : ptrs)
        if (q) cudaFree(q);
}

// Compiled kernel shapes of the chunked 2D forward (launch_forward2d_cslab)
// and variants of the staged 2D backprojector (launch_backward2d_smem): the
// defaults and the autotuner's other candidates.
constexpr int kFwdChunkShapes[] = {443, 474, 484};
constexpr int kBwdStagedVariants[] = {27, 48, 68};

template <size_t N>
bool listed(const int (&list)[N], int v) {
    for (int k : list)
        if (k == v) return true;
    return false;
}

// Overrides of a new plan's algorithms for measurement and testing, read
// from CURADON_GB300_ALGO: comma-separated key=value tokens, e.g.
// "fwd2d=tex,bwd2d_minb=48".  Keys: fwd2d = alu | tex | cslab |
// cslab<443 | 474 | 484>; bwd2d = alu | tex | smem; bwd2d_minb = 27 | 48 | 68
// (staged backprojector variants); adj2d = pair | quad; fwd3d = alu | tex3 |
// quad | mixed; fwd3d_tex = 0..8 (texture warps of 8 in the mixed forward);
// fwd3d_unroll = 1 | 2 (samples per iteration of the quad / mixed forward);
// fwd3d_block = BXxBYxBZ; bwd3d = quad | pair (general kernel on row-pair
// quads or on 8-byte pairs, its fallback where quads do not fit) | ax8m5
// (axial runs);
// adj3d = pair | quad; adj3d_order = band | view; adj3d_merge = 0 | 1;
// adj3d_agg = 0 | 1 (warp-aggregated atomics on the merged quads);
// t3d = step | exact (running-sum or drift-free sample parameters of the 3D
// ray marches).  Unknown tokens are ignored; without the variable every plan
// starts at the measured defaults.
void apply_algo_env(Plan2d *p2, Plan3d *p3) {
    const char *env = std::getenv("CURADON_GB300_ALGO");
    if (!env) return;
    std::vector<std::pair<std::string, std::string>> kv;
    {
        std::string e(env), tok;
        for (size_t i = 0; i <= e.size(); ++i) {
            if (i == e.size() || e[i] == ',') {
                const size_t eq = tok.find('=');
                if (eq != std::string::npos) kv.emplace_back(tok.substr(0, eq), tok.substr(eq + 1));
                tok.clear();
            } else {
                tok += e[i];
            }
        }
    }
    for (const auto &[key, val] : kv) {
        if (p2 && key == "fwd2d") {
            if (val == "alu") p2->algo_fwd = 0;
            if (val == "tex") p2->algo_fwd = 1;
            if (val.rfind("cslab", 0) == 0) {
                p2->algo_fwd = 4;
                for (int k : kFwdChunkShapes)
                    if (val == "cslab" + std::to_string(k)) p2->fwd_chunk_rows = k;
            }
        }
        if (p2 && key == "bwd2d") {
            if (val == "alu") p2->algo_bwd = 0;
            if (val == "tex") p2->algo_bwd = 1;
            if (val == "smem") p2->algo_bwd = 2;
        }
        if (p2 && key == "adj2d") {
            if (val == "pair") p2->adj_quad = 0;
            if (val == "quad") p2->adj_quad = 1;
        }
        if (p2 && key == "bwd2d_sym") {
            if (val == "off") p2->bwd_sym_mode = -1;
            if (val == "on") p2->bwd_sym_mode = 1;
        }
        if (p2 && key == "bwd2d_minb")
            for (int k : kBwdStagedVariants)
                if (val == std::to_string(k)) p2->bwd_min_blocks = k;
        if (p3 && key == "fwd3d") {
            if (val == "alu") p3->algo_fwd = 0;
            if (val == "tex3") p3->algo_fwd = 1;
            if (val == "quad") p3->algo_fwd = 4;
            if (val == "mixed") p3->algo_fwd = 5;
        }
        if (p3 && key == "fwd3d_unroll") {
            if (val == "1") p3->fwd_unroll = 1;
            if (val == "2") p3->fwd_unroll = 2;
        }
        if (p3 && key == "fwd3d_tex")
            for (int k = 0; k <= 8; ++k)
                if (val == std::to_string(k)) p3->fwd_tex_warps = k;
        if (p3 && key == "bwd3d") {
            if (val == "quad") p3->algo_bwd = 0, p3->bwd_packed = 3;
            if (val == "pair") p3->algo_bwd = 0, p3->bwd_packed = 2;
            if (val == "ax8m5") p3->algo_bwd = 1;
        }
        if (p3 && key == "t3d") {
            if (val == "step") p3->exact_t = false;
            if (val == "exact") p3->exact_t = true;
        }
        if (p3 && key == "adj3d_agg") p3->adj_agg = val == "1";
        if (p3 && key == "adj3d_merge") {
            if (val == "0") p3->adj_merge = false;
            if (val == "1") p3->adj_merge = true;
        }
        if (p3 && key == "adj3d_order") {
            if (val == "view") p3->adj_band = 0;
            if (val == "band") p3->adj_band = 1;
        }
        if (p3 && key == "adj3d") {
            if (val == "pair") p3->adj_quad = 0;
            if (val == "quad") p3->adj_quad = 1;
        }
        if (p3 && key == "fwd3d_block") {
            int bx = 0, by = 0, bz = 0;
            if (std::sscanf(val.c_str(), "%dx%dx%d", &bx, &by, &bz) == 3 && bx > 0 && by > 0 &&
                bz > 0 && bx * by * bz <= 1024 && bx % 8 == 0)
                p3->fwd_bx = bx, p3->fwd_by = by, p3->fwd_bz = bz;
        }
    }
}

// ------------------------------------------------------------ 3D geometry

namespace {

// Three-vector with the component-wise float operations of the reference's
// vec<f32, 3> (vec.hpp), used to evaluate the per-view geometry in the same
// FP32 operation order as the reference's host code.
struct V3 {
    float v[3];
    float &operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};
inline V3 operator+(const V3 &a, const V3 &b) { return {{a[0] + b[0], a[1] + b[1], a[2] + b[2]}}; }
inline V3 operator-(const V3 &a, const V3 &b) { return {{a[0] - b[0], a[1] - b[1], a[2] - b[2]}}; }
inline V3 operator/(const V3 &a, const V3 &b) { return {{a[0] / b[0], a[1] / b[1], a[2] / b[2]}}; }
inline V3 operator/(const V3 &a, float s) { return {{a[0] / s, a[1] / s, a[2] / s}}; }

// Y-Z-Y Euler rotation, rotation.hpp:7-28 (matrix written out there).
V3 rot_yzy(const V3 &v, float phi, float theta, float psi) {
    const float cphi = std::cos(phi), sphi = std::sin(phi);
    const float ctheta = std::cos(theta), stheta = std::sin(theta);
    const float spsi = std::sin(psi), cpsi = std::cos(psi);
    V3 r;
    r[0] = v[0] * (cphi * cpsi * ctheta - sphi * spsi) - v[1] * stheta * cphi +
           v[2] * (sphi * cpsi + spsi * cphi * ctheta);
    r[1] = v[0] * (stheta * cpsi) + v[1] * ctheta + v[2] * spsi * stheta;
    r[2] = v[0] * (-sphi * cpsi * ctheta - spsi * cphi) + v[1] * sphi * stheta +
           v[2] * (-sphi * spsi * ctheta + cpsi * cphi);
    return r;
}

// Roll-pitch-yaw rotation, rotation.hpp:31-48.
V3 rot_rpy(const V3 &v, float roll, float pitch, float yaw) {
    const float croll = std::cos(roll), sroll = std::sin(roll);
    const float cpitch = std::cos(pitch), spitch = std::sin(pitch);
    const float syaw = std::sin(yaw), cyaw = std::cos(yaw);
    V3 r;
    r[0] = croll * cpitch * v[0] + (croll * spitch * syaw - sroll * cyaw) * v[1] +
           (croll * spitch * cyaw + sroll * syaw) * v[2];
    r[1] = sroll * cpitch * v[0] + (sroll * spitch * syaw + croll * cyaw) * v[1] +
           (sroll * spitch * cyaw - croll * syaw) * v[2];
    r[2] = -spitch * v[0] + cpitch * syaw * v[1] + cpitch * cyaw * v[2];
    return r;
}

inline float4 f4(const V3 &a) { return make_float4(a[0], a[1], a[2], 0.f); }

struct Cone {
    V3 shape_f, spacing, offset;  // internal (x, y, z)
    float U, V;                   // detector cells as float (u, v)
    float su, sv, offu, offv;
    float pitch, roll, yaw, DSO, DSD, COR;
};

// Forward tables: forward_3d.hpp:117-190.
void cone_fwd_tables(const Cone &c, const float *phi, const float *theta, const float *psi,
                     int n, std::vector<float4> &org, std::vector<float4> &du,
                     std::vector<float4> &dv, std::vector<float4> &src) {
    const V3 vol_size = {{c.shape_f[0] * c.spacing[0], c.shape_f[1] * c.spacing[1],
                          c.shape_f[2] * c.spacing[2]}};
    const float DOD = c.DSD - c.DSO;
    for (int i = 0; i < n; ++i) {
        V3 s0 = {{0.f, 0.f, -c.DSO}};
        V3 o0 = {{-c.su * (c.U / 2.f) + c.su * 0.5f, -c.sv * (c.V / 2.f) + c.sv * 0.5f, 0.f}};
        V3 u0 = o0 + V3{{c.su, 0.f, 0.f}};
        V3 v0 = o0 + V3{{0.f, c.sv, 0.f}};
        o0 = rot_rpy(o0, c.roll, c.pitch, c.yaw);
        u0 = rot_rpy(u0, c.roll, c.pitch, c.yaw);
        v0 = rot_rpy(v0, c.roll, c.pitch, c.yaw);
        o0[2] += DOD;
        u0[2] += DOD;
        v0[2] += DOD;
        V3 o = rot_yzy(o0, phi[i], theta[i], psi[i]);
        V3 pu = rot_yzy(u0, phi[i], theta[i], psi[i]);
        V3 pv = rot_yzy(v0, phi[i], theta[i], psi[i]);
        V3 s = rot_yzy(s0, phi[i], theta[i], psi[i]);
        const V3 tr = vol_size / 2.f - c.spacing / 2.f;
        o = o - c.offset + tr;
        pu = pu - c.offset + tr;
        pv = pv - c.offset + tr;
        s = s - c.offset + tr;
        o = o / c.spacing;
        pu = pu / c.spacing;
        pv = pv / c.spacing;
        s = s / c.spacing;
        const float cor_x = c.COR * std::sin(phi[i]) / c.spacing[0];
        const float cor_z = c.COR * std::cos(phi[i]) / c.spacing[2];
        o[0] += cor_x, o[2] += cor_z, pu[0] += cor_x, pu[2] += cor_z;
        pv[0] += cor_x, pv[2] += cor_z, s[0] += cor_x, s[2] += cor_z;
        org.push_back(f4(o));
        du.push_back(f4(pu - o));
        dv.push_back(f4(pv - o));
        src.push_back(f4(s));
    }
}

// Backward tables: backward_3d.hpp:122-166 and the source of :218-227.
void cone_bwd_tables(const Cone &c, const float *phi, const float *theta, const float *psi,
                     int n, std::vector<float4> &org, std::vector<float4> &dx,
                     std::vector<float4> &dy, std::vector<float4> &dz, float src[3]) {
    const V3 ext = {{c.shape_f[0] * c.spacing[0], c.shape_f[1] * c.spacing[1],
                     c.shape_f[2] * c.spacing[2]}};
    const float DOD = c.DSD - c.DSO;
    const V3 neg_ext = {{-ext[0], -ext[1], -ext[2]}};
    const V3 init = neg_ext / 2.f + c.spacing / 2.f + c.offset;
    for (int i = 0; i < n; ++i) {
        auto fn = [&](V3 p) {
            p = rot_yzy(p, phi[i], theta[i], psi[i]);
            p[0] += c.offu;
            p[1] += c.offv;
            p[2] -= DOD;
            p = rot_rpy(p, c.roll, c.pitch, c.yaw);
            p[2] += DOD;
            return p;
        };
        const V3 o = fn(init);
        org.push_back(f4(o));
        V3 d = init;
        d[0] += c.spacing[0];
        dx.push_back(f4(fn(d) - o));
        d = init;
        d[1] += c.spacing[1];
        dy.push_back(f4(fn(d) - o));
        d = init;
        d[2] += c.spacing[2];
        dz.push_back(f4(fn(d) - o));
    }
    V3 s = {{-c.offu, -c.offv, -c.DSO}};
    s[2] -= DOD;
    s = rot_rpy(s, c.roll, c.pitch, c.yaw);
    s[2] += DOD;
    src[0] = s[0], src[1] = s[1], src[2] = s[2];
}

bool finite_all(const float *a, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

int check_device(int device) {
    int count = 0;
    CG_TRY_CUDA(cudaGetDeviceCount(&count));
    CG_REQUIRE(device >= 0 && device < count, "device index out of range");
    return CG_OK;
}

int make_plan3d(cg_plan3d **out, int device, const uint64_t vol_shape[3], const float vol_spacing[3],
                const float vol_offset[3], const float *phi, const float *theta,
                const float *psi, uint64_t nangles, const uint64_t det_shape[2],
                const float det_spacing[2], const float det_offset[2],
                const float det_rotation[3], float DSO, float DSD, float COR) {
    CG_REQUIRE(out, "plan output pointer is NULL");
    *out = nullptr;
    CG_REQUIRE(vol_shape && vol_spacing && vol_offset && det_shape && det_spacing && det_offset &&
                   det_rotation,
               "geometry array is NULL");
    CG_REQUIRE(nangles > 0 && phi && theta && psi, "angles are missing");
    CG_REQUIRE(nangles <= 65535, "at most 65535 views per plan");
    for (int d = 0; d < 3; ++d)
        CG_REQUIRE(vol_shape[d] > 0 && vol_shape[d] <= (1u << 16), "volume shape out of range");
    for (int d = 0; d < 2; ++d)
        CG_REQUIRE(det_shape[d] > 0 && det_shape[d] <= (1u << 16), "detector shape out of range");
    CG_REQUIRE(finite_all(phi, nangles) && finite_all(theta, nangles) && finite_all(psi, nangles),
               "angles must be finite");
    CG_REQUIRE(std::isfinite(DSO) && std::isfinite(DSD) && std::isfinite(COR),
               "DSO, DSD and COR must be finite");
    {
        int rc = check_device(device);
        if (rc) return rc;
    }
    DeviceGuard guard(device);
    CG_REQUIRE(guard.ok(), "cannot select device");

    std::unique_ptr<cg_plan3d> p(new cg_plan3d());
    p->device = device;
    // Python (z, y, x) -> internal (x, y, z); (v, u) -> (u, v) (forward.cu:47-58)
    p->X = (int)vol_shape[2], p->Y = (int)vol_shape[1], p->Z = (int)vol_shape[0];
    p->U = (int)det_shape[1], p->V = (int)det_shape[0];
    p->nangles = (int)nangles;
    p->DSO = DSO, p->DSD = DSD;
    // forward 5: 4 of 8 warps on the texture unit from 300^3 voxels (512^3:
    // -2 % against 3), 3 below (256^3 and 128^3: -2 % against 4)
    if ((long long)p->X * p->Y * p->Z >= 27000000LL) p->fwd_tex_warps = 4;
    // drift-free sample parameters where the running sum drifts measurably
    // (rays of ~900 samples and more)
    p->exact_t = std::max(p->X, std::max(p->Y, p->Z)) >= 512;
    apply_algo_env(nullptr, p.get());
    Cone c;
    c.shape_f = {{(float)vol_shape[2], (float)vol_shape[1], (float)vol_shape[0]}};
    c.spacing = {{vol_spacing[2], vol_spacing[1], vol_spacing[0]}};
    c.offset = {{vol_offset[2], vol_offset[1], vol_offset[0]}};
    c.U = (float)det_shape[1], c.V = (float)det_shape[0];
    c.su = det_spacing[1], c.sv = det_spacing[0];
    c.offu = det_offset[1], c.offv = det_offset[0];
    c.pitch = det_rotation[0], c.roll = det_rotation[1], c.yaw = det_rotation[2];
    c.DSO = DSO, c.DSD = DSD, c.COR = COR;

    std::vector<float4> fo, fu, fv, fs, bo, bx, by, bz;
    cone_fwd_tables(c, phi, theta, psi, (int)nangles, fo, fu, fv, fs);
    cone_bwd_tables(c, phi, theta, psi, (int)nangles, bo, bx, by, bz, p->bsrc);
    int rc = CG_OK;
    auto fail = [&](int code) {
        free_plan3d(p.get());
        return code;
    };
    if ((rc = alloc_copy(&p->d_forg, fo.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_fdu, fu.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_fdv, fv.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_fsrc, fs.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_borg, bo.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_bdx, bx.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_bdy, by.data(), nangles))) return fail(rc);
    if ((rc = alloc_copy(&p->d_bdz, bz.data(), nangles))) return fail(rc);
    p->axial = true;
    for (const float4 &d : by) p->axial = p->axial && d.x == 0.f && d.z == 0.f;
    if (p->axial) {
        p->ax_views.reserve(nangles * 10);
        for (uint64_t i = 0; i < nangles; ++i) {
            const float v[10] = {bo[i].x - p->bsrc[0], bo[i].y - p->bsrc[1], bo[i].z - p->bsrc[2],
                                 bx[i].x, bx[i].y, bx[i].z, bz[i].x, bz[i].y, bz[i].z, by[i].y};
            p->ax_views.insert(p->ax_views.end(), v, v + 10);
        }
    }
    *out = p.release();
    return CG_OK;
}

}  // namespace
}  // namespace cg

using namespace cg;

// ============================================================ C ABI

extern "C" {

const char *cg_last_error(void) { return g_last_error.c_str(); }

int cg_version(void) { return 1 * 10000 + 0 * 100 + 0; }

int cg_wait_timeouts(unsigned long long *count) {
    clear_error();
    CG_REQUIRE(count, "count is NULL");
    return cg::take_wait_timeouts(count);
}

namespace {

// Device buffers every 2D plan needs besides its per-view inputs.
int alloc_plan2d_buffers(cg_plan2d *p) {
    const size_t n = p->nangles;
    auto try_malloc = [&](auto **ptr, size_t elems) {
        cudaError_t e = cudaMalloc(ptr, sizeof(**ptr) * elems);
        if (e != cudaSuccess)
            return set_error(e == cudaErrorMemoryAllocation ? CG_ERR_NOMEM : CG_ERR_CUDA,
                             std::string("plan allocation: ") + cudaGetErrorString(e));
        return CG_OK;
    };
    int rc = CG_OK;
    if ((rc = try_malloc(&p->d_src, n))) return rc;
    if ((rc = try_malloc(&p->d_u0, n))) return rc;
    if ((rc = try_malloc(&p->d_du, n))) return rc;
    if (!p->vec && (rc = try_malloc(&p->d_bmeta, n))) return rc;
    if ((rc = try_malloc(&p->d_bproj, 2 * n))) return rc;
    if ((rc = try_malloc(&p->d_layA, (size_t)p->pitchA() * (p->H + 2 * kPad)))) return rc;
    if ((rc = try_malloc(&p->d_layB, (size_t)p->pitchB() * (p->W + 2 * kPad)))) return rc;
    if ((rc = try_malloc(&p->d_sinoP, (size_t)p->pitchS() * n))) return rc;
    return CG_OK;
}

double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// Tables of a vector plan, in FP64 and stored as FP32.  Per view i the six
// numbers are the source S, the detector centre C and the step U from one
// detector cell centre to the next, in the world frame of the circular plan
// (x along the volume's width; the reference's FanGeometry.to_vec layout,
// geometry.py:54-80).  Forward: the source and the direction from it to the
// centre of cell 0, C - (det - 1)/2 U, and the per-cell step U, all in voxel
// index units as plan_2d::precompute produces them.  Backprojection: the ray
// from S through a pixel P meets the detector line C + t U at
//   t = ((S - C) x (P - S)) / (U x (P - S))  cells from the centre, and the
// magnification is w = ((C - S) x U) / ((P - S) x U); for a circular view
// these are the reference's u - det/2 and DSD / (x' + DSO).
int vec_tables(cg_plan2d &p, const float *vecs, float2 *src, float2 *u0, float2 *du,
               float4 *proj) {
    const size_t n = p.nangles;
    const double half_w = 0.5 * p.W, half_h = 0.5 * p.H;
    double ds0 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const float *v = vecs + 6 * i;
        const double Sx = v[0], Sy = v[1], Cx = v[2], Cy = v[3], Ux = v[4], Uy = v[5];
        const double ds = std::hypot(Ux, Uy);
        if (i == 0) ds0 = ds;
        CG_REQUIRE(ds > 0.0, "the detector step u must be nonzero");
        // the backprojection's 1/ds factor is one number for all views, as
        // in the reference (which rejects unequal spacings, geometry.py:128)
        CG_REQUIRE(std::fabs(ds - ds0) <= 1e-5 * ds0, "the detector step must have one length");
        const double K = cross2(Cx - Sx, Cy - Sy, Ux, Uy);
        CG_REQUIRE(std::fabs(K) > 1e-9 * ds * std::hypot(Cx - Sx, Cy - Sy),
                   "the source lies on the detector line");
        const double D0x = Cx - 0.5 * (p.det - 1) * Ux, D0y = Cy - 0.5 * (p.det - 1) * Uy;
        src[i] = make_float2((float)((Sx - p.ox) / p.sx + half_w), (float)((Sy - p.oy) / p.sy + half_h));
        u0[i] = make_float2((float)((D0x - Sx) / p.sx), (float)((D0y - Sy) / p.sy));
        du[i] = make_float2((float)(Ux / p.sx), (float)(Uy / p.sy));
        // den = ((P - S) x U) / K ;  yi = -((S - C) x (P - S)) / K
        const double Ex = Sx - Cx, Ey = Sy - Cy;
        proj[i] = make_float4((float)(Uy / K), (float)(-Ux / K), (float)(-cross2(Sx, Sy, Ux, Uy) / K), 0.f);
        proj[n + i] = make_float4((float)(Ey / K), (float)(-Ex / K), (float)((Ex * Sy - Ey * Sx) / K), 0.f);
    }
    p.ds = (float)ds0;
    return CG_OK;
}

}  // namespace

namespace {

// Sets p.bwd_sym where view v + n/4 is view v turned by a quarter turn about
// the image centre and the image is large enough to gain (+1: it sees pixel (Y, -X) as view v sees (X, Y); -1: it
// sees (-Y, X)), read off the plan's projective tables: the staged
// backprojection then evaluates the geometry once for four (pixel, view)
// pairs.  Needs a square image of an even size whose pixel centres are
// symmetric about its centre; the tables must agree to 1e-5 of their
// magnitude (the views' fast sine / cosine differ in the last bits).
int detect_bwd_symmetry(Plan2d &p) {
    p.bwd_sym = 0;
    if (p.vec || p.bwd_sym_mode < 0 || p.W != p.H || (p.W & 1) || p.nangles < 4 ||
        p.nangles % 4 || p.sx != p.sy || p.ox != p.oy)
        return CG_OK;
    // a quarter of the tiles: below three blocks per SM the GPU is not
    // filled and the per-view kernel is faster (n = 512 / 1024)
    if (p.bwd_sym_mode == 0 && sym_quadrant_blocks(p.W) < 3 * sm_count()) return CG_OK;
    const float ex = (float)p.W / 2.0f;
    const float c0 = (0.f - ex) * p.sx + p.ox + 0.5f;
    const float c1 = ((float)(p.W - 1) - ex) * p.sx + p.ox + 0.5f;
    if (std::fabs(c0 + c1) > 1e-6f * std::fabs(c0)) return CG_OK;
    const int n = p.nangles, q = n / 4;
    std::vector<float4> t(2 * (size_t)n);
    CG_TRY_CUDA(cudaMemcpy(t.data(), p.d_bproj, sizeof(float4) * t.size(),
                           cudaMemcpyDeviceToHost));
    float sa = 0.f, sb = 0.f;
    for (int v = 0; v < n; ++v) {
        sa = std::max({sa, std::fabs(t[v].x), std::fabs(t[v].y)});
        sb = std::max({sb, std::fabs(t[n + v].x), std::fabs(t[n + v].y)});
    }
    constexpr float tol = 1e-5f;
    for (int dir : {1, -1}) {
        bool ok = true;
        for (int v = 0; v < n && ok; ++v) {
            const int u = (v + q) % n;
            const float4 a = t[v], a2 = t[u], b = t[n + v], b2 = t[n + u];
            const float ax = dir > 0 ? a.y : -a.y, ay = dir > 0 ? -a.x : a.x;
            const float bx = dir > 0 ? b.y : -b.y, by = dir > 0 ? -b.x : b.x;
            ok = std::fabs(a2.x - ax) <= tol * sa && std::fabs(a2.y - ay) <= tol * sa &&
                 std::fabs(a2.z - a.z) <= tol * std::fabs(a.z) &&
                 std::fabs(b2.x - bx) <= tol * sb && std::fabs(b2.y - by) <= tol * sb &&
                 std::fabs(b2.z - b.z) <= tol * sb;
        }
        if (ok) {
            p.bwd_sym = dir;
            break;
        }
    }
    return CG_OK;
}

}  // namespace

int cg_plan2d_create(cg_plan2d **plan, int device, uint32_t vol_prec, const uint64_t vol_shape[2],
                     const float vol_spacing[2], const float vol_offset[2], uint32_t det_prec,
                     uint64_t det_count, float det_spacing, float det_offset, const float *DSO,
                     const float *DSD, const float *angles, uint64_t nangles, float det_pitch,
                     float COR) {
    clear_error();
    CG_REQUIRE(plan, "plan output pointer is NULL");
    *plan = nullptr;
    // dtype_to_precision (plan.cu:20-28): 32 or 16, anything else is an error
    CG_REQUIRE((vol_prec == 32 || vol_prec == 16) && (det_prec == 32 || det_prec == 16),
               "Precision must either be f32 or f16");
    CG_REQUIRE(vol_shape && vol_spacing && vol_offset, "volume geometry array is NULL");
    CG_REQUIRE(DSO && DSD && angles, "DSO, DSD and angles must be given");
    CG_REQUIRE(nangles > 0, "at least one view is needed");
    CG_REQUIRE(nangles <= (1u << 22), "too many views");
    CG_REQUIRE(det_count > 0 && det_count <= (1u << 20), "det_count out of range");
    CG_REQUIRE(vol_shape[0] > 0 && vol_shape[1] > 0 && vol_shape[0] <= (1u << 15) &&
                   vol_shape[1] <= (1u << 15),
               "volume shape out of range");
    CG_REQUIRE(finite_all(angles, nangles) && finite_all(DSO, nangles) && finite_all(DSD, nangles),
               "angles, DSO and DSD must be finite");
    CG_REQUIRE(std::isfinite(det_spacing) && det_spacing != 0.f, "det_spacing must be nonzero");
    CG_REQUIRE(vol_spacing[0] != 0.f && vol_spacing[1] != 0.f, "vol_spacing must be nonzero");
    {
        int rc = check_device(device);
        if (rc) return rc;
    }
    DeviceGuard guard(device);
    CG_REQUIRE(guard.ok(), "cannot select device");

    std::unique_ptr<cg_plan2d> p(new cg_plan2d());
    p->device = device;
    // Python (y, x) -> internal (x, y) (plan.cu:48-50)
    p->W = (int)vol_shape[1], p->H = (int)vol_shape[0];
    p->sx = vol_spacing[1], p->sy = vol_spacing[0];
    p->ox = vol_offset[1], p->oy = vol_offset[0];
    p->det = (int)det_count, p->ds = det_spacing, p->doff = det_offset;
    p->nangles = (int)nangles, p->pitch = det_pitch, p->COR = COR;
    p->vol_bits = (int)vol_prec, p->det_bits = (int)det_prec;
    // measured on GB300 (n-sweep): the chunked forward (shape 484) takes 5 %
    // less time than the texture unit at 704^2, 11 % at 768^2, 25 % at
    // 1024^2, 39 % at 2048^2; even at 640^2, 5 % more at 512^2
    if ((long long)p->W * p->H >= 704LL * 704) p->algo_fwd = 4;
    apply_algo_env(p.get(), nullptr);
    int rc = CG_OK;
    auto fail = [&](int code) {
        free_plan2d(p.get());
        return code;
    };
    const size_t n = nangles;
    if ((rc = alloc_copy(&p->d_angles, angles, n))) return fail(rc);
    if ((rc = alloc_copy(&p->d_DSO, DSO, n))) return fail(rc);
    if ((rc = alloc_copy(&p->d_DSD, DSD, n))) return fail(rc);
    if ((rc = alloc_plan2d_buffers(p.get()))) return fail(rc);
    if ((rc = launch_plan2d_tables(*p, 0))) return fail(rc);
    {
        cudaError_t e = cudaStreamSynchronize(0);
        if (e != cudaSuccess) return fail(set_error(CG_ERR_CUDA, cudaGetErrorString(e)));
    }
    if ((rc = detect_bwd_symmetry(*p))) return fail(rc);
    *plan = p.release();
    return CG_OK;
}

int cg_plan2d_create_vec(cg_plan2d **plan, int device, uint32_t vol_prec,
                         const uint64_t vol_shape[2], const float vol_spacing[2],
                         const float vol_offset[2], uint32_t det_prec, uint64_t det_count,
                         const float *vecs, uint64_t nangles) {
    clear_error();
    CG_REQUIRE(plan, "plan output pointer is NULL");
    *plan = nullptr;
    CG_REQUIRE((vol_prec == 32 || vol_prec == 16) && (det_prec == 32 || det_prec == 16),
               "Precision must either be f32 or f16");
    CG_REQUIRE(vol_shape && vol_spacing && vol_offset && vecs, "geometry array is NULL");
    CG_REQUIRE(nangles > 0 && nangles <= (1u << 22), "nangles out of range");
    CG_REQUIRE(det_count > 0 && det_count <= (1u << 20), "det_count out of range");
    CG_REQUIRE(vol_shape[0] > 0 && vol_shape[1] > 0 && vol_shape[0] <= (1u << 15) &&
                   vol_shape[1] <= (1u << 15),
               "volume shape out of range");
    CG_REQUIRE(vol_spacing[0] != 0.f && vol_spacing[1] != 0.f, "vol_spacing must be nonzero");
    CG_REQUIRE(finite_all(vecs, 6 * nangles), "vectors must be finite");
    std::unique_ptr<cg_plan2d> p(new cg_plan2d());
    p->W = (int)vol_shape[1], p->H = (int)vol_shape[0];
    p->sx = vol_spacing[1], p->sy = vol_spacing[0];
    p->ox = vol_offset[1], p->oy = vol_offset[0];
    p->det = (int)det_count, p->nangles = (int)nangles;
    p->vol_bits = (int)vol_prec, p->det_bits = (int)det_prec;
    std::vector<float2> src(nangles), u0(nangles), du(nangles);
    std::vector<float4> proj(2 * nangles);
    {
        const int rc = vec_tables(*p, vecs, src.data(), u0.data(), du.data(), proj.data());
        if (rc) return rc;
    }
    {
        int rc = check_device(device);
        if (rc) return rc;
    }
    DeviceGuard guard(device);
    CG_REQUIRE(guard.ok(), "cannot select device");
    p->device = device;
    p->vec = true;
    if ((long long)p->W * p->H >= 704LL * 704) p->algo_fwd = 4;
    apply_algo_env(p.get(), nullptr);
    p->algo_bwd = 2;  // the staged backprojector is the one driven by the projective table
    int rc = CG_OK;
    auto fail = [&](int code) {
        free_plan2d(p.get());
        return code;
    };
    if ((rc = alloc_plan2d_buffers(p.get()))) return fail(rc);
    auto up = [&](void *dst, const void *from, size_t bytes) {
        cudaError_t e = cudaMemcpy(dst, from, bytes, cudaMemcpyHostToDevice);
        return e == cudaSuccess ? CG_OK : set_error(CG_ERR_CUDA, cudaGetErrorString(e));
    };
    if ((rc = up(p->d_src, src.data(), sizeof(float2) * nangles))) return fail(rc);
    if ((rc = up(p->d_u0, u0.data(), sizeof(float2) * nangles))) return fail(rc);
    if ((rc = up(p->d_du, du.data(), sizeof(float2) * nangles))) return fail(rc);
    if ((rc = up(p->d_bproj, proj.data(), sizeof(float4) * 2 * nangles))) return fail(rc);
    *plan = p.release();
    return CG_OK;
}

int cg_plan2d_destroy(cg_plan2d *plan) {
    clear_error();
    if (!plan) return CG_OK;
    {
        DeviceGuard guard(plan->device);
        free_plan2d(plan);
    }
    delete plan;
    return CG_OK;
}

int cg_plan2d_get_forward_block(const cg_plan2d *plan, uint64_t *bx, uint64_t *by) {
    clear_error();
    CG_REQUIRE(plan && bx && by, "NULL argument");
    *bx = (uint64_t)plan->fwd_bx, *by = (uint64_t)plan->fwd_by;
    return CG_OK;
}

int cg_plan2d_set_forward_block(cg_plan2d *plan, uint64_t bx, uint64_t by) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(bx >= 32 && bx % 32 == 0 && by >= 1 && bx * by <= 256,
               "forward block must be a multiple of 32 cells wide and at most 256 threads");
    plan->fwd_bx = (int)bx, plan->fwd_by = (int)by;
    return CG_OK;
}

int cg_plan2d_set_algorithm(cg_plan2d *plan, int forward, int backward) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(forward == -1 || forward == 0 || forward == 1 || forward == 4,
               "2D forward algorithm must be 0 (registers), 1 (texture) or 4 (chunked)");
    CG_REQUIRE(backward >= -1 && backward <= 2,
               "2D backward algorithm must be 0 (registers), 1 (texture) or 2 (staged)");
    CG_REQUIRE(!plan->vec || backward == -1 || backward == 2,
               "vector-geometry plans backproject with the staged algorithm (2)");
    if (forward >= 0) plan->algo_fwd = forward;
    if (backward >= 0) plan->algo_bwd = backward;
    return CG_OK;
}

int cg_plan2d_get_algorithm(const cg_plan2d *plan, int *forward, int *backward) {
    clear_error();
    CG_REQUIRE(plan && forward && backward, "NULL argument");
    *forward = plan->algo_fwd, *backward = plan->algo_bwd;
    return CG_OK;
}

int cg_plan2d_get_symmetry(const cg_plan2d *plan, int *quarter_turn) {
    clear_error();
    CG_REQUIRE(plan && quarter_turn, "NULL argument");
    *quarter_turn = plan->bwd_sym;
    return CG_OK;
}

int cg_plan2d_set_shapes(cg_plan2d *plan, int forward_shape, int backward_variant) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(forward_shape == -1 || listed(kFwdChunkShapes, forward_shape),
               "unknown chunked-forward shape");
    CG_REQUIRE(backward_variant == -1 || listed(kBwdStagedVariants, backward_variant),
               "unknown staged-backprojector variant");
    if (forward_shape >= 0) plan->fwd_chunk_rows = forward_shape;
    if (backward_variant >= 0) plan->bwd_min_blocks = backward_variant;
    return CG_OK;
}

int cg_plan2d_get_shapes(const cg_plan2d *plan, int *forward_shape, int *backward_variant) {
    clear_error();
    CG_REQUIRE(plan && forward_shape && backward_variant, "NULL argument");
    *forward_shape = plan->fwd_chunk_rows, *backward_variant = plan->bwd_min_blocks;
    return CG_OK;
}

int cg_plan2d_tables(const cg_plan2d *plan, float *sources, float *u_origins, float *delta_us) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    DeviceGuard guard(plan->device);
    const size_t bytes = sizeof(float2) * plan->nangles;
    if (sources) CG_TRY_CUDA(cudaMemcpy(sources, plan->d_src, bytes, cudaMemcpyDeviceToHost));
    if (u_origins) CG_TRY_CUDA(cudaMemcpy(u_origins, plan->d_u0, bytes, cudaMemcpyDeviceToHost));
    if (delta_us) CG_TRY_CUDA(cudaMemcpy(delta_us, plan->d_du, bytes, cudaMemcpyDeviceToHost));
    return CG_OK;
}

namespace {

int forward2d_f32(cg_plan2d *plan, const float *volume, float *sinogram, cudaStream_t s) {
    if (plan->algo_fwd == 1) return launch_forward2d_tex(*plan, volume, sinogram, s);
    int rc = launch_relayout2d(*plan, volume, s);
    if (rc) return rc;
    if (plan->algo_fwd == 4) return launch_forward2d_cslab(*plan, sinogram, s, plan->fwd_chunk_rows);
    return launch_forward2d(*plan, sinogram, s);
}

int backward2d_f32(cg_plan2d *plan, float *volume, const float *sinogram, cudaStream_t s) {
    if (plan->algo_bwd == 1) return launch_backward2d_tex(*plan, volume, sinogram, s);
    int rc = launch_relayout_sino2d(*plan, sinogram, s);
    if (rc) return rc;
    if (plan->algo_bwd == 2) return launch_backward2d_smem(*plan, volume, s);
    return launch_backward2d(*plan, volume, s);
}

}  // namespace

int cg_forward_2d_ex(cg_plan2d *plan, const void *volume, void *sinogram, int sino_bits,
                     void *stream) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    CG_REQUIRE(sino_bits == 32 || sino_bits == 16, "sinogram precision must be 32 or 16");
    DeviceGuard guard(plan->device);
    CG_REQUIRE(guard.ok(), "cannot select the plan's device");
    cudaStream_t s = (cudaStream_t)stream;
    const bool hv = plan->vol_bits == 16, hs = sino_bits == 16;
    if (!hv && !hs) return forward2d_f32(plan, (const float *)volume, (float *)sinogram, s);
    int rc = ensure_half_scratch(*plan, hv, hs);
    if (rc) return rc;
    const float *vol = (const float *)volume;
    if (hv) {
        if ((rc = widen_half(volume, plan->d_vol32, (long long)plan->W * plan->H, s))) return rc;
        vol = plan->d_vol32;
    }
    float *sino = hs ? plan->d_sino32 : (float *)sinogram;
    if ((rc = forward2d_f32(plan, vol, sino, s))) return rc;
    if (hs) return narrow_to_half(sino, sinogram, (long long)plan->det * plan->nangles, s);
    return CG_OK;
}

int cg_backward_2d_ex(cg_plan2d *plan, void *volume, const void *sinogram, int sino_bits,
                      void *stream) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    CG_REQUIRE(sino_bits == 32 || sino_bits == 16, "sinogram precision must be 32 or 16");
    DeviceGuard guard(plan->device);
    CG_REQUIRE(guard.ok(), "cannot select the plan's device");
    cudaStream_t s = (cudaStream_t)stream;
    const bool hv = plan->vol_bits == 16, hs = sino_bits == 16;
    if (!hv && !hs) return backward2d_f32(plan, (float *)volume, (const float *)sinogram, s);
    int rc = ensure_half_scratch(*plan, hv, hs);
    if (rc) return rc;
    const float *sino = (const float *)sinogram;
    if (hs) {
        const long long n = (long long)plan->det * plan->nangles;
        if ((rc = widen_half(sinogram, plan->d_sino32, n, s))) return rc;
        sino = plan->d_sino32;
    }
    if (!hv) return backward2d_f32(plan, (float *)volume, sino, s);
    const long long nv = (long long)plan->W * plan->H;
    CG_TRY_CUDA(cudaMemsetAsync(plan->d_vol32, 0, sizeof(float) * nv, s));
    if ((rc = backward2d_f32(plan, plan->d_vol32, sino, s))) return rc;
    return add_into_half(volume, plan->d_vol32, nv, s);
}

int cg_forward_2d(cg_plan2d *plan, const float *volume, float *sinogram, void *stream) {
    return cg_forward_2d_ex(plan, volume, sinogram, 32, stream);
}

int cg_backward_2d(cg_plan2d *plan, float *volume, const float *sinogram, void *stream) {
    return cg_backward_2d_ex(plan, volume, sinogram, 32, stream);
}

int cg_adjoint_2d(cg_plan2d *plan, float *volume, const float *sinogram, void *stream) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    CG_REQUIRE(plan->vol_bits == 32, "the matched adjoint takes float32 volumes");
    DeviceGuard guard(plan->device);
    CG_REQUIRE(guard.ok(), "cannot select the plan's device");
    return launch_adjoint2d(*plan, volume, sinogram, (cudaStream_t)stream);
}

int cg_plan3d_create(cg_plan3d **plan, int device, const uint64_t vol_shape[3],
                     const float vol_spacing[3], const float vol_offset[3], const float *phi,
                     const float *theta, const float *psi, uint64_t nangles,
                     const uint64_t det_shape[2], const float det_spacing[2],
                     const float det_offset[2], const float det_rotation[3], float DSO, float DSD,
                     float COR) {
    clear_error();
    return make_plan3d(plan, device, vol_shape, vol_spacing, vol_offset, phi, theta, psi, nangles,
                       det_shape, det_spacing, det_offset, det_rotation, DSO, DSD, COR);
}

int cg_plan3d_set_algorithm(cg_plan3d *plan, int forward, int backward) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(forward == -1 || forward == 0 || forward == 1 || forward == 4 || forward == 5,
               "3D forward algorithm must be 0 (registers), 1 (texture), 4 (quad) or 5 (mixed)");
    CG_REQUIRE(backward >= -1 && backward <= 1, "3D backward algorithm must be -1..1");
    if (forward >= 0) plan->algo_fwd = forward;
    if (backward >= 0) plan->algo_bwd = backward;
    return CG_OK;
}

int cg_plan3d_get_algorithm(const cg_plan3d *plan, int *forward, int *backward) {
    clear_error();
    CG_REQUIRE(plan && forward && backward, "NULL argument");
    *forward = plan->algo_fwd, *backward = plan->runs_axial() ? 1 : 0;
    return CG_OK;
}

int cg_plan3d_destroy(cg_plan3d *plan) {
    clear_error();
    if (!plan) return CG_OK;
    {
        DeviceGuard guard(plan->device);
        free_plan3d(plan);
    }
    delete plan;
    return CG_OK;
}

int cg_forward_3d_plan(cg_plan3d *plan, const float *volume, float *sinogram, void *stream) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    DeviceGuard guard(plan->device);
    CG_REQUIRE(guard.ok(), "cannot select the plan's device");
    if (plan->algo_fwd >= 4) return launch_forward3d_quad(*plan, volume, sinogram, (cudaStream_t)stream);
    if (plan->algo_fwd != 0) return launch_forward3d_tex(*plan, volume, sinogram, (cudaStream_t)stream);
    int rc = ensure_plan3d_scratch(*plan, true, false);
    if (rc) return rc;
    return launch_forward3d(*plan, volume, sinogram, (cudaStream_t)stream);
}

int cg_backward_3d_plan(cg_plan3d *plan, float *volume, const float *sinogram, void *stream) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    DeviceGuard guard(plan->device);
    CG_REQUIRE(guard.ok(), "cannot select the plan's device");
    int rc = ensure_plan3d_scratch(*plan, false, true);
    if (rc) return rc;
    return launch_backward3d(*plan, volume, sinogram, (cudaStream_t)stream);
}

int cg_adjoint_3d_plan(cg_plan3d *plan, float *volume, const float *sinogram, void *stream) {
    clear_error();
    CG_REQUIRE(plan, "plan is NULL");
    CG_REQUIRE(volume && sinogram, "volume and sinogram must be device pointers");
    DeviceGuard guard(plan->device);
    CG_REQUIRE(guard.ok(), "cannot select the plan's device");
    int rc = ensure_plan3d_scratch(*plan, true, false);
    if (rc) return rc;
    return launch_adjoint3d(*plan, volume, sinogram, (cudaStream_t)stream);
}

static int current_device(int *dev) {
    CG_TRY_CUDA(cudaGetDevice(dev));
    return CG_OK;
}

int cg_forward_3d(const float *x, const uint64_t vol_shape[3], const float vol_spacing[3],
                  const float vol_offset[3], float *sinogram, const float *phi,
                  const float *theta, const float *psi, uint64_t nangles,
                  const uint64_t det_shape[2], const float det_spacing[2],
                  const float det_offset[2], const float det_rotation[3], float DSO, float DSD,
                  float COR, void *stream) {
    clear_error();
    int dev = 0, rc = current_device(&dev);
    if (rc) return rc;
    cg_plan3d *p = nullptr;
    rc = make_plan3d(&p, dev, vol_shape, vol_spacing, vol_offset, phi, theta, psi, nangles,
                     det_shape, det_spacing, det_offset, det_rotation, DSO, DSD, COR);
    if (rc) return rc;
    if (p->algo_fwd >= 4) {
        rc = launch_forward3d_quad(*p, x, sinogram, (cudaStream_t)stream);
    } else if (p->algo_fwd != 0) {
        rc = launch_forward3d_tex(*p, x, sinogram, (cudaStream_t)stream);
    } else {
        rc = ensure_plan3d_scratch(*p, true, false);
        if (!rc) rc = launch_forward3d(*p, x, sinogram, (cudaStream_t)stream);
    }
    // The transient plan's memory is released once the stream has used it.
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (!rc && e != cudaSuccess) rc = set_error(CG_ERR_CUDA, cudaGetErrorString(e));
    free_plan3d(p);
    delete p;
    return rc;
}

int cg_backward_3d(float *x, const uint64_t vol_shape[3], const float vol_spacing[3],
                   const float vol_offset[3], const float *sinogram, const float *phi,
                   const float *theta, const float *psi, uint64_t nangles,
                   const uint64_t det_shape[2], const float det_spacing[2],
                   const float det_offset[2], const float det_rotation[3], float DSO, float DSD,
                   float COR, void *stream) {
    clear_error();
    int dev = 0, rc = current_device(&dev);
    if (rc) return rc;
    cg_plan3d *p = nullptr;
    rc = make_plan3d(&p, dev, vol_shape, vol_spacing, vol_offset, phi, theta, psi, nangles,
                     det_shape, det_spacing, det_offset, det_rotation, DSO, DSD, COR);
    if (rc) return rc;
    rc = ensure_plan3d_scratch(*p, false, true);
    if (!rc) rc = launch_backward3d(*p, x, sinogram, (cudaStream_t)stream);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (!rc && e != cudaSuccess) rc = set_error(CG_ERR_CUDA, cudaGetErrorString(e));
    free_plan3d(p);
    delete p;
    return rc;
}

int cg_filter_rows(const float *in, float *out, const float *h, const float *pre, uint64_t nrows,
                   uint64_t ncols, float scale, void *stream) {
    clear_error();
    CG_REQUIRE(in && out && h, "in, out and h must be device pointers");
    CG_REQUIRE(in != out, "out must not alias in");
    CG_REQUIRE(ncols > 0 && ncols <= 29056, "ncols out of range (1..29056)");
    CG_REQUIRE(nrows > 0 && nrows <= (1u << 26), "nrows out of range");
    CG_REQUIRE(ceil_div((long long)nrows, 1) <= 65535LL * 8, "too many rows for one launch");
    return launch_filter_rows(in, out, h, pre, (int)nrows, (int)ncols, scale,
                              (cudaStream_t)stream);
}

}  // extern "C"
