// batch.cu -- many 2D problems per launch.
//
// Serving and iterative reconstruction run many small and medium problems
// (n = 128 .. 1024) whose single launches leave most of the 152 SMs idle and
// pay a launch each.  A batch binds a list of 2D plans to their volumes and
// sinograms once; then each direction of the whole batch is two launches
// (re-layout + operator) over a (problem, tile) work list, whatever the
// number, sizes and geometries of the problems.  Bound buffers make the
// calls stream-ordered and capturable in a CUDA graph (an iteration loop is
// captured once and replayed).
//
// The batched forward is the texture-unit ray march (algorithm 1; each
// problem's volume is copied into its plan's array, then one launch samples
// all problems through their bindless texture handles), or, selected with
// cg_batch2d_set_forward, the FP32 register march (algorithm 0) or each
// plan's own default (algorithm 2: the chunked shared-memory forward for
// problems from 704^2 pixels, one re-layout and one bundle launch over all
// of them, and the texture march for the rest); the batched
// backprojection is the staged one (algorithm 2); cg_batch2d_adjoint runs
// the matched adjoint (the exact transpose of the register march) over the
// same work list.  Each problem uses its own
// plan's scratch, so a plan may appear in one batch only once, and a batch
// must not overlap on the GPU with other calls on its plans.
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "common.cuh"

struct cg_batch2d {
    int device = 0;
    int count = 0;
    int fwd_algo = 1;  // 1 texture unit, 0 registers, 2 each plan's own (chunked / texture)
    std::vector<cg::Plan2d *> plans;
    std::vector<cg::Prob2d> probs;  // host copy (the texture forward's copies)
    cg::Prob2d *d_probs = nullptr;
    int *d_starts = nullptr;  // kBatchStages stages x (count + 1)
    int totals[cg::kBatchStages] = {};
    std::vector<int> starts;  // host copy of d_starts
    int active = 0;           // problems [0, active) run (cg_batch2d_set_active)
    bool adjoint_ready = false;  // the plans' quad accumulators are bound

    // blocks of each stage for the active problems
    void active_totals(int out[cg::kBatchStages]) const {
        for (int st = 0; st < cg::kBatchStages; ++st) out[st] = starts[st * (count + 1) + active];
    }
};

// A 3D batch: the quad forward (with each plan's texture warps) and the
// backprojection (axial runs where the plan takes them, else the general
// kernel on row-pair quads) of every problem over one work list.
struct cg_batch3d {
    int device = 0;
    int count = 0;
    int active = 0;
    std::vector<cg::Plan3d *> plans;
    std::vector<cg::Prob3d> probs;
    cg::Prob3d *d_probs = nullptr;
    int *d_starts = nullptr;  // kBatch3dStages stages x (count + 1)
    std::vector<int> starts;
    float *d_ax = nullptr;  // axial view tables of every problem
    bool adjoint_ready = false;  // the plans' quad accumulators are bound

    void active_totals(int out[cg::kBatch3dStages]) const {
        for (int st = 0; st < cg::kBatch3dStages; ++st)
            out[st] = starts[st * (count + 1) + active];
    }
};

using namespace cg;

namespace {

void free_batch(cg_batch2d *b) {
    if (b->d_probs) cudaFree(b->d_probs);
    if (b->d_starts) cudaFree(b->d_starts);
}

// floats of a problem's axial view tables (10 per view), rounded up so that
// every problem's float4 tables start on 16 bytes
size_t ax_stride(const Plan3d &p) { return ((size_t)p.nangles * 10 + 3) & ~size_t(3); }

void free_batch3d(cg_batch3d *b) {
    if (b->d_probs) cudaFree(b->d_probs);
    if (b->d_starts) cudaFree(b->d_starts);
    if (b->d_ax) cudaFree(b->d_ax);
}

}  // namespace

extern "C" {

int cg_batch2d_create(cg_batch2d **batch, cg_plan2d *const *plans, float *const *volumes,
                      float *const *sinograms, int count) {
    clear_error();
    CG_REQUIRE(batch, "batch output pointer is NULL");
    *batch = nullptr;
    CG_REQUIRE(plans && volumes && sinograms, "plan, volume and sinogram lists must be given");
    CG_REQUIRE(count > 0 && count <= (1 << 20), "count out of range");
    std::set<const cg_plan2d *> seen;
    for (int i = 0; i < count; ++i) {
        CG_REQUIRE(plans[i] && volumes[i] && sinograms[i], "NULL plan or buffer in the batch");
        CG_REQUIRE(plans[i]->device == plans[0]->device, "all plans of a batch share one device");
        CG_REQUIRE(plans[i]->vol_bits == 32, "batches take float32 plans");
        CG_REQUIRE(seen.insert(plans[i]).second, "a plan appears twice in one batch");
    }
    DeviceGuard guard(plans[0]->device);
    CG_REQUIRE(guard.ok(), "cannot select the plans' device");

    std::vector<Prob2d> probs(count);
    std::vector<int> starts(kBatchStages * (count + 1), 0);
    long long totals[kBatchStages] = {};
    for (int i = 0; i < count; ++i) {
        const Plan2d &p = *plans[i];
        Prob2d &q = probs[i];
        q.vol = volumes[i], q.sino = sinograms[i];
        q.src = p.d_src, q.u0 = p.d_u0, q.du = p.d_du, q.bproj = p.d_bproj;
        q.layA = p.d_layA, q.layB = p.d_layB, q.sinoP = p.d_sinoP;
        q.W = p.W, q.H = p.H, q.det = p.det, q.nangles = p.nangles;
        q.pa = p.pitchA(), q.pb = p.pitchB();
        q.sx = p.sx, q.sy = p.sy, q.ox = p.ox, q.oy = p.oy, q.ds = p.ds;
        if (int rc = ensure_vol_texture(*plans[i])) return rc;
        q.tex = p.tex_vol, q.arr = p.arr_vol;
        q.quadA = p.d_quadA, q.quadB = p.d_quadB;
        q.chunked = batch_chunked(p) ? 1 : 0;
        q.bwd_sym = p.bwd_sym;
        int blocks[kBatchStages];
        batch_blocks(p, blocks);
        for (int st = 0; st < kBatchStages; ++st) {
            starts[st * (count + 1) + i] = (int)totals[st];
            totals[st] += blocks[st];
            starts[st * (count + 1) + i + 1] = (int)totals[st];
        }
    }
    // stages 7..9 hold only the problems of one kind of the "plans" forward
    // and may be empty; the others have blocks for every problem
    for (long long t : totals)
        CG_REQUIRE(t < (1ll << 31), "batch too large for one launch");

    std::unique_ptr<cg_batch2d> b(new cg_batch2d());
    b->device = plans[0]->device;
    b->count = count;
    b->active = count;
    b->starts = starts;
    b->plans.assign(plans, plans + count);
    b->probs = probs;
    for (int st = 0; st < kBatchStages; ++st) b->totals[st] = (int)totals[st];
    auto fail = [&](cudaError_t e) {
        free_batch(b.get());
        return set_error(e == cudaErrorMemoryAllocation ? CG_ERR_NOMEM : CG_ERR_CUDA,
                         std::string("batch set-up: ") + cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaMalloc(&b->d_probs, sizeof(Prob2d) * count)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_starts, sizeof(int) * starts.size())) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpy(b->d_probs, probs.data(), sizeof(Prob2d) * count,
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e);
    if ((e = cudaMemcpy(b->d_starts, starts.data(), sizeof(int) * starts.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e);
    *batch = b.release();
    return CG_OK;
}

int cg_batch2d_destroy(cg_batch2d *batch) {
    clear_error();
    if (!batch) return CG_OK;
    {
        DeviceGuard guard(batch->device);
        free_batch(batch);
    }
    delete batch;
    return CG_OK;
}

int cg_batch2d_forward(cg_batch2d *batch, void *stream) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    DeviceGuard guard(batch->device);
    CG_REQUIRE(guard.ok(), "cannot select the batch's device");
    int totals[kBatchStages];
    batch->active_totals(totals);
    if (batch->fwd_algo == 1)
        return launch_batch2d_fwd_tex(batch->d_probs, batch->probs, batch->active,
                                      batch->d_starts + (batch->count + 1), totals[1],
                                      (cudaStream_t)stream);
    if (batch->fwd_algo == 2)
        return launch_batch2d_fwd_plans(batch->d_probs, batch->probs, batch->active,
                                        batch->d_starts, totals, batch->count,
                                        (cudaStream_t)stream);
    return launch_batch2d(batch->d_probs, batch->d_starts, totals, batch->count, true,
                          (cudaStream_t)stream);
}

int cg_batch2d_set_active(cg_batch2d *batch, int active) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    CG_REQUIRE(active > 0 && active <= batch->count, "active count must be in [1, count]");
    batch->active = active;
    return CG_OK;
}

int cg_batch2d_set_forward(cg_batch2d *batch, int algorithm) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    CG_REQUIRE(algorithm >= 0 && algorithm <= 2, "batched forward algorithm must be 0, 1 or 2");
    batch->fwd_algo = algorithm;
    return CG_OK;
}

int cg_batch2d_get_forward(const cg_batch2d *batch, int *algorithm) {
    clear_error();
    CG_REQUIRE(batch && algorithm, "NULL argument");
    *algorithm = batch->fwd_algo;
    return CG_OK;
}

int cg_batch2d_adjoint(cg_batch2d *batch, void *stream) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    DeviceGuard guard(batch->device);
    CG_REQUIRE(guard.ok(), "cannot select the batch's device");
    if (!batch->adjoint_ready) {
        // first call: every plan's quad accumulators, bound into the work list
        for (int i = 0; i < batch->count; ++i) {
            if (int rc = ensure_adj2d_quads(*batch->plans[i])) return rc;
            batch->probs[i].quadA = batch->plans[i]->d_quadA;
            batch->probs[i].quadB = batch->plans[i]->d_quadB;
        }
        CG_TRY_CUDA(cudaMemcpy(batch->d_probs, batch->probs.data(),
                               sizeof(Prob2d) * batch->count, cudaMemcpyHostToDevice));
        batch->adjoint_ready = true;
    }
    int totals[kBatchStages];
    batch->active_totals(totals);
    return launch_batch2d_adjoint(batch->d_probs, batch->d_starts, totals, batch->count,
                                  (cudaStream_t)stream);
}

int cg_batch2d_backward(cg_batch2d *batch, void *stream) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    DeviceGuard guard(batch->device);
    CG_REQUIRE(guard.ok(), "cannot select the batch's device");
    int totals[kBatchStages];
    batch->active_totals(totals);
    return launch_batch2d(batch->d_probs, batch->d_starts, totals, batch->count, false,
                          (cudaStream_t)stream);
}

int cg_batch3d_create(cg_batch3d **batch, cg_plan3d *const *plans, float *const *volumes,
                      float *const *sinograms, int count) {
    clear_error();
    CG_REQUIRE(batch, "batch output pointer is NULL");
    *batch = nullptr;
    CG_REQUIRE(plans && volumes && sinograms, "plan, volume and sinogram lists must be given");
    CG_REQUIRE(count > 0 && count <= (1 << 20), "count out of range");
    std::set<const cg_plan3d *> seen;
    size_t ax_floats = 0;
    for (int i = 0; i < count; ++i) {
        CG_REQUIRE(plans[i] && volumes[i] && sinograms[i], "NULL plan or buffer in the batch");
        CG_REQUIRE(plans[i]->device == plans[0]->device, "all plans of a batch share one device");
        CG_REQUIRE(seen.insert(plans[i]).second, "a plan appears twice in one batch");
        ax_floats += ax_stride(*plans[i]);
    }
    DeviceGuard guard(plans[0]->device);
    CG_REQUIRE(guard.ok(), "cannot select the plans' device");

    std::unique_ptr<cg_batch3d> b(new cg_batch3d());
    b->device = plans[0]->device;
    b->count = count;
    b->active = count;
    b->plans.assign(plans, plans + count);
    auto fail = [&](cudaError_t e) {
        free_batch3d(b.get());
        return set_error(e == cudaErrorMemoryAllocation ? CG_ERR_NOMEM : CG_ERR_CUDA,
                         std::string("batch set-up: ") + cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaMalloc(&b->d_ax, ax_floats * sizeof(float))) != cudaSuccess) return fail(e);
    std::vector<Prob3d> probs(count);
    std::vector<int> starts(kBatch3dStages * (count + 1), 0);
    long long totals[kBatch3dStages] = {};
    size_t ax_off = 0;
    for (int i = 0; i < count; ++i) {
        int blocks[kBatch3dStages];
        if (int rc = bind_batch3d_problem(*plans[i], volumes[i], sinograms[i], b->d_ax + ax_off,
                                          &probs[i], blocks)) {
            free_batch3d(b.get());
            return rc;
        }
        ax_off += ax_stride(*plans[i]);
        for (int st = 0; st < kBatch3dStages; ++st) {
            starts[st * (count + 1) + i] = (int)totals[st];
            totals[st] += blocks[st];
            starts[st * (count + 1) + i + 1] = (int)totals[st];
        }
    }
    for (long long t : totals)
        if (t >= (1ll << 31)) {
            free_batch3d(b.get());
            return set_error(CG_ERR_INVALID, "batch too large for one launch");
        }
    b->probs = probs;
    b->starts = starts;
    if ((e = cudaMalloc(&b->d_probs, sizeof(Prob3d) * count)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_starts, sizeof(int) * starts.size())) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpy(b->d_probs, probs.data(), sizeof(Prob3d) * count,
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e);
    if ((e = cudaMemcpy(b->d_starts, starts.data(), sizeof(int) * starts.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e);
    *batch = b.release();
    return CG_OK;
}

int cg_batch3d_destroy(cg_batch3d *batch) {
    clear_error();
    if (!batch) return CG_OK;
    {
        DeviceGuard guard(batch->device);
        free_batch3d(batch);
    }
    delete batch;
    return CG_OK;
}

int cg_batch3d_set_active(cg_batch3d *batch, int active) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    CG_REQUIRE(active > 0 && active <= batch->count, "active count must be in [1, count]");
    batch->active = active;
    return CG_OK;
}

int cg_batch3d_forward(cg_batch3d *batch, void *stream) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    DeviceGuard guard(batch->device);
    CG_REQUIRE(guard.ok(), "cannot select the batch's device");
    const cudaStream_t s = (cudaStream_t)stream;
    // the texture warps' volumes into their plans' arrays, then the work list
    for (int i = 0; i < batch->active; ++i)
        if (batch->probs[i].tex_warps > 0)
            if (int rc = upload_volume_texture3(*batch->plans[i], batch->probs[i].vol, s))
                return rc;
    int totals[kBatch3dStages];
    batch->active_totals(totals);
    return launch_batch3d_forward(batch->d_probs, batch->d_starts, totals, batch->count, s);
}

int cg_batch3d_adjoint(cg_batch3d *batch, void *stream) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    DeviceGuard guard(batch->device);
    CG_REQUIRE(guard.ok(), "cannot select the batch's device");
    if (!batch->adjoint_ready) {
        // first call: every plan's quad accumulators, bound into the work list
        for (int i = 0; i < batch->count; ++i) {
            if (int rc = ensure_adj3d_quads(*batch->plans[i])) return rc;
            batch->probs[i].adjA = batch->plans[i]->d_quadA;
            batch->probs[i].adjB = batch->plans[i]->d_quadB;
        }
        CG_TRY_CUDA(cudaMemcpy(batch->d_probs, batch->probs.data(),
                               sizeof(Prob3d) * batch->count, cudaMemcpyHostToDevice));
        batch->adjoint_ready = true;
    }
    int totals[kBatch3dStages];
    batch->active_totals(totals);
    return launch_batch3d_adjoint(batch->d_probs, batch->d_starts, totals, batch->count,
                                  (cudaStream_t)stream);
}

int cg_batch3d_backward(cg_batch3d *batch, void *stream) {
    clear_error();
    CG_REQUIRE(batch, "batch is NULL");
    DeviceGuard guard(batch->device);
    CG_REQUIRE(guard.ok(), "cannot select the batch's device");
    int totals[kBatch3dStages];
    batch->active_totals(totals);
    return launch_batch3d_backward(batch->d_probs, batch->d_starts, totals, batch->count,
                                   (cudaStream_t)stream);
}

}  // extern "C"
