/*
 * curadon_gb300.h -- C ABI of the GB300 (sm_103a) projection operators.
 *
 * Drop-in boundary for curadon's native extension `curadon_ext`
 * (python/standalone/src/bind.cpp:58-66 of the reference).  Every entry point
 * below replaces one function of that extension and keeps its argument
 * meaning; reference locations are given beside each declaration.
 *
 * Conventions
 *  - All data pointers are CUDA device pointers to C-contiguous float32
 *    arrays; geometry arrays are host pointers.
 *  - Python axis order is used for shapes, as in the reference's bindings:
 *      2D volume (H, W), 2D sinogram (nangles, det_count);
 *      3D volume (Z, Y, X), 3D sinogram (nangles, V, U).
 *  - Work is enqueued on `stream` (a cudaStream_t, NULL = legacy default
 *    stream) and is asynchronous; nothing synchronises the host.
 *  - Every function returns CG_OK or an error code; the message of the last
 *    error on the calling thread is returned by cg_last_error().  No function
 *    aborts the process (the reference's gpuErrchk exits; error.h:6-18).
 *  - Forward projections overwrite the sinogram (2D: every ray; 3D: every ray
 *    that hits the volume's bounding box, as forward_3d.hpp:74-76 skips the
 *    others).  Backprojections ADD into the volume, as the reference does
 *    (backward_2d.hpp:99, backward_3d.hpp:44-53 and :98-106).
 *  - A plan's geometry is fixed at creation; its selectors (algorithm,
 *    kernel shape, forward block shape) may change between calls, not while a
 *    call on the plan is in flight.  One plan may be used from several threads
 *    on different streams, but two calls on the same plan must not overlap on
 *    the GPU (they share the plan's scratch).
 */
#ifndef CURADON_GB300_H
#define CURADON_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_OK 0
#define CG_ERR_INVALID 1     /* bad argument: null pointer, shape, size      */
#define CG_ERR_CUDA 2        /* a CUDA runtime call or launch failed         */
#define CG_ERR_NOMEM 3       /* device allocation failed                     */
#define CG_ERR_UNSUPPORTED 4 /* valid in the reference, not built here       */

/* Message of the last failed call on this thread ("" if none). */
const char *cg_last_error(void);

/* ABI version: major * 10000 + minor * 100 + patch. */
int cg_version(void);

/* Number of bounded waits (on asynchronous copies) that gave up in this
 * library's kernels on the current device since the last call, which the
 * call then clears.  Every wait in a kernel has an iteration limit so that a
 * lost copy cannot hang the GPU; a nonzero count means results computed
 * since the last call are not to be trusted.  No reference counterpart. */
int cg_wait_timeouts(unsigned long long *count);

/* ------------------------------------------------------------------ 2D -- */

typedef struct cg_plan2d cg_plan2d;

/* Fan-beam plan.  Replaces `plan_2d.__init__` (plan.cu:20-59) and the
 * plan_2d constructor (plan_2d.hpp:103-126): per-view source, detector origin
 * and detector step are precomputed on the device exactly as
 * plan_2d::precompute does (plan_2d.hpp:189-241), and the scratch the
 * operators need is allocated here, once.  vol_prec / det_prec are bit widths
 * (32 or 16, plan.cu:20-28): vol_prec is the element type of every volume
 * passed with this plan (float or IEEE half); det_prec is recorded, and the
 * sinogram's type is given per call, as the reference reads it from the array.
 * vol_shape / vol_spacing / vol_offset are in Python order (y, x).
 * det_pitch and COR are accepted and, as in the reference, unused. */
int cg_plan2d_create(cg_plan2d **plan, int device, uint32_t vol_prec,
                     const uint64_t vol_shape[2], const float vol_spacing[2],
                     const float vol_offset[2], uint32_t det_prec, uint64_t det_count,
                     float det_spacing, float det_offset, const float *DSO, const float *DSD,
                     const float *angles, uint64_t nangles, float det_pitch, float COR);

/* Fan-beam plan from per-view vectors: vecs holds nangles x 6 floats
 * [source.x, source.y, detector_centre.x, detector_centre.y, u.x, u.y] in
 * the layout of the reference's FanGeometry.to_vec / from_vec
 * (geometry.py:54-134; x along the volume's width, u the step from one
 * detector cell centre to the next).  The reference reduces such vectors to
 * angles / DSO / DSD (from_vec, losing per-view shifts of source and
 * detector); this plan keeps them: the forward marches the rays the vectors
 * define and the backprojection maps each pixel through the view's own
 * projective map.  For vectors made by to_vec from a circular geometry the
 * results equal cg_plan2d_create's within FP32 rounding.  All views must
 * share one |u| (the detector spacing).  The backprojection uses the staged
 * algorithm (2).  No counterpart call in the reference. */
int cg_plan2d_create_vec(cg_plan2d **plan, int device, uint32_t vol_prec,
                         const uint64_t vol_shape[2], const float vol_spacing[2],
                         const float vol_offset[2], uint32_t det_prec, uint64_t det_count,
                         const float *vecs, uint64_t nangles);

/* Frees the plan and its device memory (plan_2d destructor). */
int cg_plan2d_destroy(cg_plan2d *plan);

/* The reference's read-write `forward_block_x` / `forward_block_y`
 * (plan.cu:57-58, plan_2d.hpp:184-186): here they set the detector-cells x
 * views shape of one forward thread block (x a multiple of 32, x * y <= 256). */
int cg_plan2d_get_forward_block(const cg_plan2d *plan, uint64_t *bx, uint64_t *by);
int cg_plan2d_set_forward_block(cg_plan2d *plan, uint64_t bx, uint64_t by);

/* Algorithm of each operator of a plan; -1 leaves one unchanged; other
 * values are rejected with CG_ERR_INVALID.
 *   forward:  0 registers (FP32 filtering of pair-packed copies, gathered
 *               through L1), 1 texture unit, 4 chunked shared-memory slabs
 *   backward: 0 registers, 1 texture unit, 2 shared-memory detector windows
 * The texture unit filters with 8-bit weight fractions, exactly as the
 * reference does; the other algorithms filter in FP32, and cg_adjoint_2d is
 * the transpose of forward algorithms 0 and 4 (exact for 0; 4 takes the
 * same samples and weights, summed in another order).  A new plan starts
 * at the fastest measured combination: forward 4 from 704^2 pixels, else 1;
 * backward 2. */
int cg_plan2d_set_algorithm(cg_plan2d *plan, int forward, int backward);
int cg_plan2d_get_algorithm(const cg_plan2d *plan, int *forward, int *backward);

/* Whether the staged backprojection (algorithm 2) of this plan runs over
 * the views' quarter-turn symmetry: *quarter_turn = +1 / -1 where view
 * v + nangles/4 is view v turned by +-90 degrees about the image centre
 * (same DSO / DSD, square image of an even size with centred pixels; found
 * on the plan's tables at creation) and the image is large enough for its
 * first quadrant's 32 x 32-pixel tiles to give every SM three blocks, else
 * 0.  One projective evaluation then serves the four (pixel, view) pairs
 * the turn relates; results differ from the per-view evaluation only by
 * the last bits of the views' tables (relative L2 ~3e-6 at n = 2048).
 * CURADON_GB300_ALGO=bwd2d_sym=off / on overrides the size rule. */
int cg_plan2d_get_symmetry(const cg_plan2d *plan, int *quarter_turn);

/* Kernel shape of the chunked forward (forward algorithm 4) and variant of
 * the staged backprojector (backward algorithm 2); -1 keeps the current one.
 * Shapes: 443, 474, 484 (default); variants: 27, 48, 68 (default).  Every
 * shape computes the reference's samples and weights; they differ in rows
 * per chunk, pair layout, staging and warp layout, so the fastest depends
 * on the geometry (no reference counterpart: the reference has one kernel
 * per direction, forward_2d.hpp:21-79 and backward_2d.hpp:21-100).  Where
 * the backprojection runs over the views' quarter-turn symmetry
 * (cg_plan2d_get_symmetry) the variant has no effect.  Used by the
 * autotuner (curadon_gb300.autotune).  CG_ERR_INVALID for an unknown
 * shape. */
int cg_plan2d_set_shapes(cg_plan2d *plan, int forward_shape, int backward_variant);
int cg_plan2d_get_shapes(const cg_plan2d *plan, int *forward_shape, int *backward_variant);

/* Copies the plan's per-view tables to host arrays of 2 * nangles floats each
 * (x, y interleaved): source position, direction to detector cell 0 and
 * per-cell step, in voxel-index units (plan_2d::sources/u_origins/delta_us,
 * plan_2d.hpp:174-182).  Any pointer may be NULL. */
int cg_plan2d_tables(const cg_plan2d *plan, float *sources, float *u_origins, float *delta_us);

/* 2D ray-driven forward projection.  Replaces `forward_2d(volume, sinogram,
 * plan)` (forward.cu:92-139 -> fp::forward_2d, forward_2d.hpp:135-139) for a
 * float32 sinogram; `volume` holds the plan's vol_prec. */
int cg_forward_2d(cg_plan2d *plan, const float *volume, float *sinogram, void *stream);

/* 2D voxel-driven backprojection, accumulating into `volume`.  Replaces
 * `backward_2d(volume, sinogram, plan)` (backward.cu:89-133 ->
 * bp::backproject_2d, backward_2d.hpp:162-166) for a float32 sinogram. */
int cg_backward_2d(cg_plan2d *plan, float *volume, const float *sinogram, void *stream);

/* The same two operators with the sinogram's element type given: sino_bits
 * 32 (float) or 16 (IEEE half); the volume's is the plan's vol_prec.  These
 * are the four typed instantiations of forward_2d_cuda_typed /
 * backward_2d_cuda_typed (forward.cu:77-135, backward.cu:75-135).  Half data
 * is widened to FP32, every computation is FP32, a half sinogram gets each
 * ray sum rounded to nearest and a half volume gets half(acc / ds) added in
 * half arithmetic, as the reference's kernels store to __half. */
int cg_forward_2d_ex(cg_plan2d *plan, const void *volume, void *sinogram, int sino_bits,
                     void *stream);
int cg_backward_2d_ex(cg_plan2d *plan, void *volume, const void *sinogram, int sino_bits,
                      void *stream);

/* Matched adjoint of cg_forward_2d, accumulating A^T sinogram into `volume`:
 * the exact transpose of the ray-driven interpolation (same rays, sample
 * points and weights), for gradients and solvers that need <Ax,y> = <x,A^T y>.
 * No counterpart call in the reference, whose backward of the forward is the
 * voxel-driven backprojector (diffable.py:21-24).  float32 plans only. */
int cg_adjoint_2d(cg_plan2d *plan, float *volume, const float *sinogram, void *stream);

/* ------------------------------------------------------------------ 3D -- */

typedef struct cg_plan3d cg_plan3d;

/* Cone-beam plan: the argument list of the reference's per-call
 * `forward_3d` / `backward_3d` (forward.cu:23-38, backward.cu:20-35), held
 * once so the per-view geometry (forward_3d.hpp:97-211,
 * backward_3d.hpp:110-178) is computed and uploaded once.
 *   vol_shape/vol_spacing/vol_offset: Python order (z, y, x)
 *   phi/theta/psi: per-view Euler angles, `nangles` each.  `phi` is the
 *     array the reference receives in its 6th position (curadon.forward
 *     passes geom.angles[0]) and uses as phi (forward.cu:60-66).
 *   det_shape/det_spacing/det_offset: Python order (v, u)
 *   det_rotation: (pitch, roll, yaw) */
int cg_plan3d_create(cg_plan3d **plan, int device, const uint64_t vol_shape[3],
                     const float vol_spacing[3], const float vol_offset[3], const float *phi,
                     const float *theta, const float *psi, uint64_t nangles,
                     const uint64_t det_shape[2], const float det_spacing[2],
                     const float det_offset[2], const float det_rotation[3], float DSO, float DSD,
                     float COR);
int cg_plan3d_destroy(cg_plan3d *plan);

/* Algorithm of each 3D operator; -1 leaves one unchanged; other values are
 * rejected with CG_ERR_INVALID.
 *   forward:  0 registers (FP32 trilinear from pair-packed copies),
 *             1 texture unit (tex3D),
 *             4 quads (FP32 trilinear, two 16-byte loads per sample),
 *             5 quads with 3 of every 8 warps (4 from 300^3 voxels) on the
 *             texture unit (default)
 *   backward: 0 registers (voxel runs along z), 1 runs along y when every
 *             view maps the volume's y axis onto the detector's v axis
 *             (circular orbits without detector tilt; default), else 0.
 * cg_plan3d_get_algorithm reports the backward algorithm that runs.
 * cg_adjoint_3d_plan is the transpose of forward algorithms 0 and 4 (the
 * same samples and trilinear weights, up to FP32 rounding). */
int cg_plan3d_set_algorithm(cg_plan3d *plan, int forward, int backward);
int cg_plan3d_get_algorithm(const cg_plan3d *plan, int *forward, int *backward);

/* 3D ray-driven forward projection with a plan (fp::forward_3d,
 * forward_3d.hpp:214-274). */
int cg_forward_3d_plan(cg_plan3d *plan, const float *volume, float *sinogram, void *stream);

/* 3D voxel-driven backprojection with a plan, accumulating
 * (bp::backproject_3d, backward_3d.hpp:181-253). */
int cg_backward_3d_plan(cg_plan3d *plan, float *volume, const float *sinogram, void *stream);

/* Matched adjoint of cg_forward_3d_plan, accumulating into `volume`; rays
 * that miss the volume contribute nothing.  No counterpart in the reference
 * (see cg_adjoint_2d). */
int cg_adjoint_3d_plan(cg_plan3d *plan, float *volume, const float *sinogram, void *stream);

/* Per-call forms with the reference's exact argument list: they build a
 * transient plan (as the reference allocates its texture array per call),
 * run, and release it once the stream has finished with it.
 * Replace `forward_3d(...)` (forward.cu:23-75) and `backward_3d(...)`
 * (backward.cu:20-72). */
int cg_forward_3d(const float *x, const uint64_t vol_shape[3], const float vol_spacing[3],
                  const float vol_offset[3], float *sinogram, const float *phi,
                  const float *theta, const float *psi, uint64_t nangles,
                  const uint64_t det_shape[2], const float det_spacing[2],
                  const float det_offset[2], const float det_rotation[3], float DSO, float DSD,
                  float COR, void *stream);
int cg_backward_3d(float *x, const uint64_t vol_shape[3], const float vol_spacing[3],
                   const float vol_offset[3], const float *sinogram, const float *phi,
                   const float *theta, const float *psi, uint64_t nangles,
                   const uint64_t det_shape[2], const float det_spacing[2],
                   const float det_offset[2], const float det_rotation[3], float DSO, float DSD,
                   float COR, void *stream);

/* 2D backprojection that allocates nothing, for callers that cannot call
 * cudaMalloc (a server whose device memory is reserved up front by its own
 * pool, a real-time loop that must not wait on or fail in the allocator, a
 * plugin host that forbids allocations by the libraries it loads).  It has no
 * counterpart in the reference.  Same result as cg_plan2d_create +
 * cg_backward_2d on the same arguments (plan_2d's geometry without
 * det_offset, which the backprojection does not use), accumulating into
 * `volume`; all scratch lives in one 16 MiB device array that the library
 * holds on every GPU that loads it.  A call needs at most
 * 8 * nangles * (det_count + 4) + 84 * nangles + 2040 bytes of it; larger
 * problems are rejected with CG_ERR_INVALID.  Each call looks the array's
 * device address up in the current context and copies `angles`, `DSO` and
 * `DSD` from (pageable) host memory with cudaMemcpyAsync on `stream`, so a
 * call cannot be captured into a CUDA graph.  All calls share the array:
 * calls that overlap on the GPU race and must be ordered by the caller. */
int cg_backward_2d_static(float *volume, const float *sinogram, const uint64_t vol_shape[2],
                          const float vol_spacing[2], const float vol_offset[2],
                          uint64_t det_count, float det_spacing, const float *DSO,
                          const float *DSD, const float *angles, uint64_t nangles,
                          void *stream);

/* ----------------------------------------------------------------- FBP -- */

/* Row filter of filtered backprojection: out[r][k] = scale * sum_j
 * pre[j] * in[r][j] * h[(k - j) mod ncols] for each of the nrows rows, i.e. the
 * circular convolution that the reference's FBP evaluates through the FFT
 * (examples/fbp.py:51-56: multiply each row's DFT by a real response and
 * keep the real part; h is the real part of that response's inverse DFT).
 * in, out, h (ncols floats) and pre (ncols floats, or NULL for none) are
 * device pointers; out must not alias in.  ncols <= 29056. */
int cg_filter_rows(const float *in, float *out, const float *h, const float *pre, uint64_t nrows,
                   uint64_t ncols, float scale, void *stream);

/* ------------------------------------------------------------- batches -- */

/* A batch binds `count` float32 2D plans (any sizes and geometries, each
 * plan at most once) to their device volumes and sinograms.  Each direction
 * of the whole batch then runs as two launches over a (problem, tile) work
 * list instead of two launches per problem: the serving / many-problem entry
 * point, capturable in a CUDA graph because the buffers are bound.  The
 * batched forward is the texture-unit ray march (algorithm 1, default: one
 * array copy per problem, then one launch) or the register ray march
 * (algorithm 0: a re-layout launch and one launch), the batched
 * backprojection the staged one (algorithm 2); results equal cg_forward_2d /
 * cg_backward_2d with those algorithms bit for bit.  A batch must not run
 * concurrently with other calls on its plans.  No counterpart call in the
 * reference, which runs one problem per call. */
typedef struct cg_batch2d cg_batch2d;
int cg_batch2d_create(cg_batch2d **batch, cg_plan2d *const *plans, float *const *volumes,
                      float *const *sinograms, int count);
int cg_batch2d_destroy(cg_batch2d *batch);
/* sinogram_i = A_i volume_i for every problem (overwrites the sinograms) */
int cg_batch2d_forward(cg_batch2d *batch, void *stream);
/* volume_i += A_i^T sinogram_i for every problem */
int cg_batch2d_backward(cg_batch2d *batch, void *stream);
/* volume_i += the matched adjoint (exact transpose of the register ray
 * march, cg_adjoint_2d's operator) of sinogram_i for every problem, as three
 * launches over the work list (zeroing, scatter, fold).  Pairs with the
 * batched forward on algorithm 0 for gradients and solvers that need A^T.
 * The first call allocates the plans' accumulators (make it before any
 * stream capture).  No counterpart in the reference, whose gradient is its
 * backprojector (python/standalone/src/curadon/diffable.py:14-38). */
int cg_batch2d_adjoint(cg_batch2d *batch, void *stream);
/* Later forward / backward / adjoint calls run only problems [0, active)
 * of the batch (1 <= active <= count; all of them after creation): a
 * resident batch of `count` slots serves however many requests are waiting
 * without being rebuilt. */
int cg_batch2d_set_active(cg_batch2d *batch, int active);
/* the batched forward's algorithm: 1 texture unit (default), 0 registers,
 * 2 each plan's own default (the chunked shared-memory forward for problems
 * from 704^2 pixels, the texture unit below; results equal cg_forward_2d on
 * the plans bit for bit) */
int cg_batch2d_set_forward(cg_batch2d *batch, int algorithm);
int cg_batch2d_get_forward(const cg_batch2d *batch, int *algorithm);

/* The same for 3D: `count` plans (any volume and detector sizes, views and
 * geometries, each plan at most once) bound to their device volumes and
 * projections.  The forward is three launches over the work list (the two
 * quad re-layouts of every volume, then the quad ray march of every
 * problem, with each plan's texture warps: algorithm 5 plans first copy
 * their volume into the plan's array), the backprojection two or three
 * (the projections' re-layout, then axial runs for the problems whose plan
 * takes them and the general kernel on row-pair quads for the others).
 * Results equal cg_forward_3d_plan on plans with forward algorithm 4 or 5
 * (algorithm 4 for plans set to 0 or 1) and cg_backward_3d_plan bit for
 * bit; as there, the forward writes only the rays that hit the volume's box
 * and the backprojection adds into the volumes.  Creation allocates each
 * plan's quad copies (4 x 16 bytes per padded voxel and per padded
 * projection cell) and fails with CG_ERR_NOMEM where they do not fit.  No
 * counterpart in the reference (forward_3d.hpp:97-211 and
 * backward_3d.hpp:110-178 run one problem per call). */
typedef struct cg_batch3d cg_batch3d;
int cg_batch3d_create(cg_batch3d **batch, cg_plan3d *const *plans, float *const *volumes,
                      float *const *sinograms, int count);
int cg_batch3d_destroy(cg_batch3d *batch);
int cg_batch3d_forward(cg_batch3d *batch, void *stream);
int cg_batch3d_backward(cg_batch3d *batch, void *stream);
/* volume_i += the matched adjoint (cg_adjoint_3d_plan's operator, the exact
 * transpose of the quad forward without texture warps) of projections_i for
 * every problem, as three launches over the work list (zeroing, scatter,
 * fold); equal to cg_adjoint_3d_plan up to the order of its atomic
 * additions.  Pairs with a batch of plans on forward algorithm 4.  The first
 * call allocates the plans' accumulators (make it before any stream
 * capture).  No counterpart in the reference, whose gradient is its
 * backprojector (python/standalone/src/curadon/diffable.py:14-38). */
int cg_batch3d_adjoint(cg_batch3d *batch, void *stream);
/* later calls run problems [0, active) only, as cg_batch2d_set_active */
int cg_batch3d_set_active(cg_batch3d *batch, int active);

#ifdef __cplusplus
}
#endif

#endif /* CURADON_GB300_H */
