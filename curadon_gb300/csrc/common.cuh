// common.cuh -- error reporting, plan structures and small device helpers
// shared by the sm_103a projection kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "curadon_gb300.h"

namespace cg {

// ------------------------------------------------------------ error state

// Records `msg` as this thread's last error and returns `code`.
int set_error(int code, const std::string &msg);
void clear_error();

#define CG_TRY_CUDA(expr)                                                                     \
    do {                                                                                      \
        cudaError_t cg_err_ = (expr);                                                         \
        if (cg_err_ != cudaSuccess) {                                                         \
            return ::cg::set_error(cg_err_ == cudaErrorMemoryAllocation ? CG_ERR_NOMEM        \
                                                                        : CG_ERR_CUDA,        \
                                   std::string(#expr) + ": " + cudaGetErrorName(cg_err_) +    \
                                       " (" + cudaGetErrorString(cg_err_) + ")");             \
        }                                                                                     \
    } while (0)

#define CG_REQUIRE(cond, msg)                                                                 \
    do {                                                                                      \
        if (!(cond)) return ::cg::set_error(CG_ERR_INVALID, (msg));                           \
    } while (0)

// Runs `expr` on the plan's device and restores the caller's device after.
class DeviceGuard {
  public:
    explicit DeviceGuard(int device) {
        cudaGetDevice(&prev_);
        if (prev_ != device) {
            ok_ = cudaSetDevice(device) == cudaSuccess;
            switched_ = true;
        }
    }
    ~DeviceGuard() {
        if (switched_) cudaSetDevice(prev_);
    }
    bool ok() const { return ok_; }

  private:
    int prev_ = 0;
    bool switched_ = false;
    bool ok_ = true;
};

// Padding, in texels, around the pair-packed copies of volumes and
// sinograms.  Sample coordinates are clamped into the padded range, whose
// outer texels are zero, which reproduces the texture unit's border mode.
constexpr int kPad = 2;

// ------------------------------------------------------------ plan types

struct Plan2d {
    int device = 0;
    int W = 0, H = 0;                 // internal x (contiguous), y
    float sx = 1, sy = 1, ox = 0, oy = 0;
    int det = 0;
    float ds = 1, doff = 0;
    int nangles = 0;
    float pitch = 0, COR = 0;
    int fwd_bx = 32, fwd_by = 8;

    // per-view tables (device)
    float *d_angles = nullptr, *d_DSO = nullptr, *d_DSD = nullptr;
    float2 *d_src = nullptr, *d_u0 = nullptr, *d_du = nullptr;
    float4 *d_bmeta = nullptr;        // (-sin, cos, DSD, DSO)
    // backprojection as a projective map per view, 2 x nangles entries:
    // [i] = (ax, ay, a0, -), [n + i] = (bx, by, b0, -); for the pixel's world
    // position (X, Y): w = 1 / (ax X + ay Y + a0), u = (bx X + by Y + b0) w + det/2
    float4 *d_bproj = nullptr;
    bool vec = false;                 // per-view vectors (no angles / DSO / DSD)

    // scratch (device)
    float2 *d_layA = nullptr;         // (H+2P) rows x pitchA() pairs along x
    float2 *d_layB = nullptr;         // (W+2P) rows x pitchB() pairs along y
    float2 *d_sinoP = nullptr;        // nangles x (det+2P) pairs along u

    // FP16 storage: precisions of the volume (plan) and FP32 staging of half
    // data (allocated on first use)
    int vol_bits = 32, det_bits = 32;
    float *d_vol32 = nullptr, *d_sino32 = nullptr;

    // matched adjoint: quad accumulators (float4 per padded texel of layA /
    // layB), allocated on first use; adj_quad -1 = when both fit in 96 MB,
    // 1 = always, 0 = never (pair accumulators in layA / layB)
    float4 *d_quadA = nullptr, *d_quadB = nullptr;
    int adj_quad = -1;

    // texture-unit variants (allocated on first use)
    cudaArray_t arr_vol = nullptr, arr_sino = nullptr;
    cudaTextureObject_t tex_vol = 0, tex_sino = 0;

    // algorithm per operator: forward 0 = registers, 1 = texture unit,
    // 4 = chunked shared-memory slabs; backprojection 0 = registers,
    // 1 = texture unit, 2 = staged shared-memory windows.  Defaults: the
    // fastest measured on GB300 (2D n-sweep); the forward becomes chunked for
    // volumes of 704^2 pixels and more (cg_plan2d_create).
    int algo_fwd = 1, algo_bwd = 2;
    // chunked forward's kernel shape: 484 (default: 16-row chunks staged by
    // bulk copies on mbarriers, bundles of 8 views x 128 cells, two threads
    // per cell on 4 interleaved views, packed sums, absolute-position pairs),
    // 474 (the same staged by per-lane cp.async) or 443 ((v, d) pairs, pair
    // reuse, view groups four views apart); the autotuner's candidates
    int fwd_chunk_rows = 484;
    // staged backprojector's variant: 68 (default: packed FP32 row pairs,
    // floor by FP32 adds, window rows by bulk copies, absolute-position
    // pairs, 8 x 4-pixel warps), 48 (the same staged pair by pair with
    // cp.async) or 27 ((t, d) pairs, 32 x 1-pixel warps); the autotuner's
    // candidates
    int bwd_min_blocks = 68;
    // staged backprojection over the views' quarter-turn symmetry: +1 / -1
    // when view v + nangles/4 is view v turned by +-90 degrees about the
    // image centre (checked on the plan's tables at creation), square
    // centred pixels; 0 otherwise or where disabled
    int bwd_sym = 0;
    // CURADON_GB300_ALGO bwd2d_sym=off / on: never, or wherever the geometry
    // has the symmetry (default: where the first quadrant's tiles give every
    // SM at least three blocks)
    int bwd_sym_mode = 0;

    // row pitches of layA / layB in pairs, even so every row starts on 16 bytes
    int pitchA() const { return (W + 2 * kPad + 1) & ~1; }
    int pitchB() const { return (H + 2 * kPad + 1) & ~1; }
    int pitchS() const { return det + 2 * kPad; }
};

// One problem of a 2D batch as the batched kernels see it.
struct Prob2d {
    float *vol;    // volume: forward input, backprojection accumulator
    float *sino;   // sinogram: forward output, backprojection input
    const float2 *src, *u0, *du;
    const float4 *bproj;
    float2 *layA, *layB, *sinoP;
    int W, H, det, nangles, pa, pb;
    float sx, sy, ox, oy, ds;
    cudaTextureObject_t tex;  // the plan's volume texture (texture forward)
    cudaArray_t arr;          // and its array
    float4 *quadA, *quadB;    // matched adjoint: the plan's quad accumulators
    int chunked;              // the batched "plans" forward runs the chunked kernel
    int bwd_sym;              // the plan's quarter-turn symmetry (Plan2d::bwd_sym)
};

// Problem of a batched launch's block b: the last i with start[i] <= b
// (stage s of problem i owns the blocks [start[i], start[i + 1])).
__device__ __forceinline__ int batch_problem(const int *__restrict__ start, int count, int b) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}
// One problem of a 3D batch as the batched kernels see it (a bound plan's
// buffers and tables).
struct Prob3d {
    float *vol;   // volume: forward input, backprojection accumulator
    float *sino;  // projections: forward output, backprojection input
    // forward: the plan's quad copies and tables; texture warps per block
    float4 *QA, *QB;
    const float4 *forg, *fdu, *fdv, *fsrc;
    cudaTextureObject_t tex;
    int tex_warps, exact_t;
    int X, Y, Z, U, V, P, utiles;
    // backprojection: the re-laid projections (quads of rows v, v + 1)
    float4 *sinoQ;
    int axial;  // runs along y (k_bwd3d_ax) or the general kernel
    // axial: per-view tables (p0, p1, p2 as the kernel parameter holds them)
    // and the constant terms; general: the plan's tables and source
    const float4 *ax0, *ax1;
    const float2 *ax2;
    float num, su, sv;
    const float4 *borg, *bdx, *bdy, *bdz;
    float bsx, bsy, bsz, zplane, hu, hv;
    int tiles_x, tiles_y, tiles_z;
    // matched adjoint: the plan's quad accumulators (bound on first use)
    float4 *adjA, *adjB;
};
// 3D batch stages: the two volume quad re-layouts, the forward, the
// projections' re-layout, the axial and the general backprojection, the
// matched adjoint's zeroing, scatter and fold
constexpr int kBatch3dStages = 9;

// Batched stages: re-layout, forward, sinogram re-layout, backprojection,
// the matched adjoint's zeroing, scatter and fold, the "plans" forward's
// absolute-position re-layout and chunked bundles (chunked problems) and
// texture rays (the others), and the backprojection over the quarter-turn
// symmetry (problems whose plan has it; stage 3 holds the others).
constexpr int kBatchStages = 11;
// chunked-forward shape the batched "plans" forward compiles
constexpr int kBatchChunkShape = 484;

struct Plan3d {
    int device = 0;
    int X = 0, Y = 0, Z = 0;          // internal volume extents (x fastest)
    int U = 0, V = 0;                 // detector cells (u fastest)
    int nangles = 0;
    float DSO = 0, DSD = 0;

    // forward tables: detector origin, u step, v step, source (voxel units)
    float4 *d_forg = nullptr, *d_fdu = nullptr, *d_fdv = nullptr, *d_fsrc = nullptr;
    // backward tables: voxel (0,0,0) origin, x/y/z steps (world units)
    float4 *d_borg = nullptr, *d_bdx = nullptr, *d_bdy = nullptr, *d_bdz = nullptr;
    float bsrc[3] = {0, 0, 0};        // backward source (same for all views)

    // scratch (device), allocated on first use
    float2 *d_volA = nullptr;         // (Z+2P)(Y+2P)(X+2P) pairs along x
    float2 *d_volB = nullptr;         // (X+2P)(Y+2P)(Z+2P) pairs along z
    float2 *d_sinoP = nullptr;        // nangles (V+2P)(U+2P) pairs along u
    float4 *d_sinoQ = nullptr;        // quads of rows v, v+1 (backward 1; 0 variant 3)
    float4 *d_volQA = nullptr;        // forward 4: quads, slices z (Z+kQP)(Y+kQP)(X+kQP)
    float4 *d_volQB = nullptr;        // forward 4: quads, slices x (X+kQP)(Y+kQP)(Z+kQP)
    size_t volA_elems = 0, volB_elems = 0, sinoP_elems = 0;
    // matched adjoint: quad accumulators (float4 per padded voxel), on first
    // use; adj_quad -1 / 1 = quads (measured faster at every size), 0 = pair
    // accumulators
    float4 *d_quadA = nullptr, *d_quadB = nullptr;
    int adj_quad = -1;
    // block order of the scatter: -1 band-major when the accumulators exceed
    // 96 MB (they no longer stay in L2), else view-major; 1 / 0 forced
    int adj_band = -1;
    // merge consecutive samples' shared quad element into one atomic
    // (-11 % at 128^3, -10 % at 256^3)
    bool adj_merge = true;
    // merged quads plus warp-aggregated atomics (lanes whose lower-slice
    // element coincides combine before one atomic)
    bool adj_agg = false;
    // ray-march sample parameters t_k = tmin + k h by one FMA instead of the
    // reference's running sum t += h, whose rounding accumulates along long
    // rays (on from 512 voxels along an axis: against the FP64 oracle the
    // running sum leaves rays of a 512^3 volume up to 2.5e-3 off, relative)
    bool exact_t = false;

    // texture-unit forward (allocated on first use)
    cudaArray_t arr3 = nullptr;
    cudaTextureObject_t tex3 = 0;

    // forward 0 = registers, 1 = tex3D, 4 = quads (FP32 trilinear, two
    // 16-byte loads per sample), 5 = quads with some warps on the texture
    // unit; backward 0 = general voxel runs along z, 1 = runs along y when
    // every view maps y onto the detector's v axis (`axial`; otherwise 0
    // runs).  Defaults: the fastest measured on GB300 (256^3 and 512^3)
    int algo_fwd = 5, algo_bwd = 1;
    // backward 0: 3 = each bilinear sample one 16-byte load of a row-pair
    // quad (default), 2 = two 8-byte pairs (where the quads do not fit)
    int bwd_packed = 3;
    // forward 5: warps of each 8 that sample through the texture unit (4 for
    // volumes of 300^3 voxels and more, set at plan creation)
    int fwd_tex_warps = 3;
    // forward 4 / 5: samples per loop iteration with their loads issued
    // together (2, default; 1); the results do not depend on it
    int fwd_unroll = 2;
    bool axial = false;  // every backward table's y step is (0, dy, 0)
    // axial backprojection, per view: source -> voxel (0, 0, 0) (3), x step
    // (3), z step (3), y step's v component (1)
    std::vector<float> ax_views;
    bool runs_axial() const { return algo_bwd == 1 && axial; }
    bool reads_quads() const { return runs_axial() || bwd_packed == 3; }
    // texture forwards: detector cells (u, v) x views per thread block
    int fwd_bx = 8, fwd_by = 4, fwd_bz = 8;
};

void free_plan2d(Plan2d *p);
void free_plan3d(Plan3d *p);

// ------------------------------------------------------------ kernels

int launch_plan2d_tables(Plan2d &p, cudaStream_t s);
int launch_relayout2d(const Plan2d &p, const float *vol, cudaStream_t s);
// Reads and clears the count of bounded waits that gave up in this
// library's kernels on the current device (cg_wait_timeouts).
int take_wait_timeouts(unsigned long long *count);
bool cslab_abs(int rows);
bool bwd_abs(int min_blocks);
int launch_forward2d(const Plan2d &p, float *sino, cudaStream_t s);
// Raises a kernel's dynamic shared-memory limit to `bytes` on the current
// device, once per (device, kernel): later calls, e.g. inside a CUDA-graph
// capture, make no runtime call.
int ensure_smem_attr(const void *func, int bytes);

// FP16 storage (half.cu)
int ensure_half_scratch(Plan2d &p, bool vol, bool sino);
int widen_half(const void *in, float *out, long long n, cudaStream_t s);
int narrow_to_half(const float *in, void *out, long long n, cudaStream_t s);
int add_into_half(void *vol, const float *add, long long n, cudaStream_t s);

int launch_relayout_sino2d(const Plan2d &p, const float *sino, cudaStream_t s);
// batches (proj2d.cu): blocks of each stage of one problem, and the launch of
// one direction over a batch whose starts hold 4 x (count + 1) block starts
void batch_blocks(const Plan2d &p, int blocks[kBatchStages]);
// true where the batched "plans" forward runs the plan's chunked shape
bool batch_chunked(const Plan2d &p);
int launch_batch2d(const Prob2d *probs, const int *starts, const int totals[kBatchStages],
                   int count, bool forward, cudaStream_t s);
// the matched adjoint's padded accumulator sizes (float4 elements) and
// their allocation (on first use)
size_t adj2d_quad_elems(const Plan2d &p, bool layoutA);
int ensure_adj2d_quads(Plan2d &p);
int launch_batch2d_adjoint(const Prob2d *probs, const int *starts,
                           const int totals[kBatchStages], int count, cudaStream_t s);
// the "plans" forward: texture rays of the problems that are not chunked
// (stage 9, after their array copies) and the chunked bundles of the others
// (stages 7 and 8), the first `active` problems
int launch_batch2d_fwd_plans(const Prob2d *d_probs, const std::vector<Prob2d> &probs,
                             int active, const int *starts, const int totals[kBatchStages],
                             int count, cudaStream_t s);
int launch_batch2d_fwd_tex_stage(const Prob2d *d_probs, const std::vector<Prob2d> &probs,
                                 int active, const int *starts, int total, bool only_unchunked,
                                 cudaStream_t s);
int launch_backward2d(const Plan2d &p, float *vol, cudaStream_t s);

int ensure_plan3d_scratch(Plan3d &p, bool fwd, bool bwd);
int launch_forward3d(const Plan3d &p, const float *vol, float *sino, cudaStream_t s);
int launch_forward3d_quad(Plan3d &p, const float *vol, float *sino, cudaStream_t s);
int launch_backward3d(const Plan3d &p, float *vol, const float *sino, cudaStream_t s);

int launch_adjoint2d(Plan2d &p, float *vol, const float *sino, cudaStream_t s);
int launch_adjoint3d(Plan3d &p, float *vol, const float *sino, cudaStream_t s);

int launch_backward2d_smem(const Plan2d &p, float *vol, cudaStream_t s);
// blocks of the quarter-turn backprojection of a W x W image
int sym_quadrant_blocks(int W);
int sm_count();
// rows: the chunked forward's compiled shape (kFwdChunkShapes: 443, 474,
// 484); views [v0, v0 + nv), all by default
int launch_forward2d_cslab(const Plan2d &p, float *sino, cudaStream_t s, int rows, int v0 = 0,
                           int nv = -1);
// The plan's 2D volume texture array and object (allocated once).
int ensure_vol_texture(Plan2d &p);
// the first `active` problems of a batch (the work list's blocks [0, total))
int launch_batch2d_fwd_tex(const Prob2d *d_probs, const std::vector<Prob2d> &probs, int active,
                           const int *starts, int total, cudaStream_t s);
int launch_forward2d_tex(Plan2d &p, const float *vol, float *sino, cudaStream_t s);
int launch_backward2d_tex(Plan2d &p, float *vol, const float *sino, cudaStream_t s);
// texture forward (tex3D, the reference's trilinear sampling)
int launch_forward3d_tex(Plan3d &p, const float *vol, float *sino, cudaStream_t s);
int upload_volume_texture3(Plan3d &p, const float *vol, cudaStream_t s);
// the plan's 3D texture array and object, without a copy
int ensure_volume_texture3(Plan3d &p);

// 3D batches (proj3d.cu): a plan bound as a batch problem (its quad scratch
// allocated; `ax` holds 10 floats of device memory per view for the axial
// tables), each stage's blocks, and the two directions over the first
// problems whose blocks are the totals
int bind_batch3d_problem(Plan3d &p, float *vol, float *sino, float *ax, Prob3d *q,
                         int blocks[kBatch3dStages]);
int launch_batch3d_forward(const Prob3d *d_probs, const int *starts,
                           const int totals[kBatch3dStages], int count, cudaStream_t s);
int launch_batch3d_backward(const Prob3d *d_probs, const int *starts,
                            const int totals[kBatch3dStages], int count, cudaStream_t s);
// the matched adjoint (adjoint.cu): the plan's quad accumulators (allocated
// on first use) and the zeroing, scatter and fold stages over a batch
int ensure_adj3d_quads(Plan3d &p);
int launch_batch3d_adjoint(const Prob3d *d_probs, const int *starts,
                           const int totals[kBatch3dStages], int count, cudaStream_t s);

// Reads CURADON_GB300_ALGO ("fwd2d=tex,bwd2d=smem,fwd3d=tex2l,...") over the
// defaults of a new plan.
void apply_algo_env(Plan2d *p2, Plan3d *p3);

int launch_filter_rows(const float *in, float *out, const float *h, const float *pre, int nrows,
                       int N, float scale, cudaStream_t s);

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// floor(x) with two FP32 adds instead of the conversion unit (which runs
// floor and float<->int conversions at a fraction of the FMA rate):
// x - 1/2 + 1.5 * 2^23 rounds to the nearest integer, which is floor(x); at
// an exact integer it may be x - 1 with fraction 1, which gives the same
// linear interpolation of a difference-encoded pair (v, next - v).  frac =
// x - floor(x); idx = floor(x) - base as an unsigned offset for the caller to
// clamp: for |x| >= 2^22, infinities and NaN it lands far outside any buffer
// and the clamp sends it to the zero padding.
struct FloorSplit {
    float frac;
    unsigned idx;
};
__device__ __forceinline__ FloorSplit floor_split(float x, int base) {
    constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
    const float t = __fadd_rn(__fadd_rn(x, -0.5f), kMagic);
    const float k = __fadd_rn(t, -kMagic);
    return {__fadd_rn(x, -k), __float_as_uint(t) - (0x4B400000u + (unsigned)base)};
}

// ---- bulk copies by the tensor-memory-access unit, completed on an mbarrier
// (PTX cp.async.bulk / mbarrier, sm_90 and later).  Addresses are 32-bit
// shared-window addresses.
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
// makes the barriers' initialisation visible to the asynchronous proxy
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// orders this thread's earlier shared-memory accesses before later bulk copies
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// the barrier's one expected arrival, announcing `bytes` of copies
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
                 : "memory");
}
// global -> shared copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned), counted against the barrier's transaction bytes
__device__ __forceinline__ void bulk_copy_g2s(unsigned dst, const void *src, unsigned bytes,
                                              unsigned bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
            "r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
// waits for the barrier's phase `parity` to complete, at most `limit` tries;
// false when it gave up
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit) {
    for (int i = 0; i < limit; ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
// Sample parameter of ray-march step k + 1: the reference's running sum t + h
// (forward_3d.hpp:85-92), or with `exact` tmin + (k + 1) h by one FMA, so
// that no rounding accumulates along the ray.
__device__ __forceinline__ float march_next(float t, int k, float tmin, float h, bool exact) {
    return exact ? fmaf((float)(k + 1), h, tmin) : t + h;
}

// 1 / x by the hardware's approximate reciprocal alone (PTX rcp.approx.ftz:
// one special-function instruction, relative error within 2^-22.9, subnormal
// results flushed to zero), for per-sample perspective weights whose
// denominators are well inside the normal range.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

}  // namespace cg

// C-ABI handles are the plan structures themselves.
struct cg_plan2d : cg::Plan2d {};
struct cg_plan3d : cg::Plan3d {};
