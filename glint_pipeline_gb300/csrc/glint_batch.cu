/*
 * glint_batch.cu -- the batching form: many independent regions advanced
 * together on one GPU.  The reference runs one region per process
 * (tracing/process.cpp:401-462); here every region is a context of its own
 * (its schema, meeting table, store, stream) inside one batch.
 *
 * A timestep of the batch is one CUDA graph, captured at the first step and
 * replayed after.  Its shape:
 *
 *   batch stream ── fork ──> region r: counters, points, partition, filter,
 *                                      refine work items            (all r)
 *                <── join ──
 *   batch stream: one refine launch over the items of every region in the
 *                 FP32-screen form (k_refine_fp32_batch)
 *                ── fork ──> region r: refine pairs (plain-form regions),
 *                                      insert, identify, keys, schema
 *                                      update on its side stream, tail,
 *                                      counters to the host        (all r)
 *                <── join ──
 *
 * The fronts and backs of small regions, which alone would leave most of the
 * GPU idle, run side by side; the refine stage, where the regions' work is
 * most uneven (a dense region has thousands of long cross-leaf lists, a
 * sparse one a few), is one pool of items that every SM drains.  Replaying
 * one graph costs one launch per timestep, not one per region.
 */
#include <algorithm>
#include <cstring>
#include <vector>

#include "glint_internal.cuh"
#include "refine_common.cuh"

struct glint_batch {
    std::vector<glint_ctx *> regions;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork_ev = nullptr, mid_ev = nullptr;
    std::vector<cudaEvent_t> front_ev, back_ev, pre_ev;
    /* the regions in the FP32-screen form: their refine arguments, the
     * per-region item offsets and the item cursor of the batched launch */
    std::vector<uint32_t> screened;
    glint::RefineArgs *d_args = nullptr;
    uint32_t *d_off = nullptr; /* ex_off[R + 1], wk_off[R + 1] */
    unsigned int *d_next = nullptr;
    uint32_t cap_max = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<const double *> src;
    bool launched = false;
    int device = 0;
};

namespace {

void batch_release(glint_batch *b) {
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto v : {&b->front_ev, &b->back_ev, &b->pre_ev})
        for (cudaEvent_t e : *v)
            if (e) cudaEventDestroy(e);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->mid_ev) cudaEventDestroy(b->mid_ev);
    cudaFree(b->d_args);
    cudaFree(b->d_off);
    cudaFree(b->d_next);
    if (b->stream) cudaStreamDestroy(b->stream);
    for (glint_ctx *c : b->regions) glint_destroy(c);
    delete b;
}

/* the launches of one timestep of every region, on the batch stream and the
 * regions' streams; captured into the batch's graph */
void launch_batch_step(glint_batch *b, const double *const *d_points) {
    const size_t R = b->regions.size();
    cudaEventRecord(b->fork_ev, b->stream);
    for (size_t r = 0; r < R; ++r) {
        glint_ctx *c = b->regions[r];
        cudaStreamWaitEvent(c->stream, b->fork_ev, 0);
        glint::launch_step_front(c, d_points[r], false);
        cudaEventRecord(b->front_ev[r], c->stream);
        cudaStreamWaitEvent(b->stream, b->front_ev[r], 0);
    }
    const uint32_t S = (uint32_t)b->screened.size();
    if (S) glint::launch_refine_precision_batch(b->d_args, S, b->cap_max, b->d_off, b->d_off + S + 1, b->d_next,
                                                b->stream);
    cudaEventRecord(b->mid_ev, b->stream);
    for (size_t r = 0; r < R; ++r) {
        glint_ctx *c = b->regions[r];
        cudaStreamWaitEvent(c->stream, b->mid_ev, 0);
        if (c->cfg.precision_mode != 1) glint::launch_refine_pairs(c);
        glint::launch_step_back(c);
        cudaEventRecord(b->back_ev[r], c->stream);
        cudaStreamWaitEvent(b->stream, b->back_ev[r], 0);
    }
}

glint_status batch_fail(glint_batch *b, cudaError_t e, const char *what) {
    for (glint_ctx *c : b->regions) c->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return GLINT_ERR_CUDA;
}

} // namespace

extern "C" glint_status glint_batch_create(uint32_t n, const glint_config *cfgs, const glint_box *mbrs,
                                           const double *const *first_points, glint_batch **out) {
    if (!out || n == 0 || !cfgs || !mbrs || !first_points) return GLINT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    glint_batch *b = new glint_batch();
    for (uint32_t r = 0; r < n; ++r) {
        glint_config cfg = cfgs[r];
        cfg.use_graph = 0; /* the batch captures the whole timestep */
        cfg.timing = 0;
        if (r > 0 && cfg.device != cfgs[0].device) {
            batch_release(b);
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        glint_ctx *c = nullptr;
        const glint_status st = glint_create(&cfg, &mbrs[r], first_points[r], nullptr, &c);
        if (st != GLINT_OK) {
            batch_release(b);
            return st;
        }
        b->regions.push_back(c);
    }
    b->device = b->regions[0]->device;
    cudaSetDevice(b->device);
    std::vector<glint::RefineArgs> args;
    for (uint32_t r = 0; r < n; ++r) {
        glint_ctx *c = b->regions[r];
        if (c->cfg.precision_mode != 1) continue;
        b->screened.push_back(r);
        args.push_back(glint::refine_args(c));
        b->cap_max = std::max(b->cap_max, c->cap);
    }
    const size_t S = b->screened.size();
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->mid_ev, cudaEventDisableTiming);
    for (auto v : {&b->front_ev, &b->back_ev, &b->pre_ev}) {
        v->assign(n, nullptr);
        for (uint32_t r = 0; r < n && e == cudaSuccess; ++r) e = cudaEventCreateWithFlags(&(*v)[r], cudaEventDisableTiming);
    }
    if (e == cudaSuccess && S) {
        e = cudaMalloc((void **)&b->d_args, sizeof(glint::RefineArgs) * S);
        if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_off, sizeof(uint32_t) * 2 * (S + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_next, sizeof(unsigned int));
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_args, args.data(), sizeof(glint::RefineArgs) * S, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        const glint_status st = batch_fail(b, e, "batch create");
        batch_release(b);
        return st;
    }
    *out = b;
    return GLINT_OK;
}

extern "C" glint_status glint_batch_destroy(glint_batch *b) {
    if (!b) return GLINT_OK;
    cudaSetDevice(b->device);
    batch_release(b);
    return GLINT_OK;
}

extern "C" uint32_t glint_batch_regions(const glint_batch *b) { return b ? (uint32_t)b->regions.size() : 0u; }

extern "C" glint_ctx *glint_batch_region(glint_batch *b, uint32_t r) {
    return (b && r < b->regions.size()) ? b->regions[r] : nullptr;
}

extern "C" glint_status glint_batch_step(glint_batch *b, const double *const *d_points, uint32_t cur_time) {
    if (!b || !d_points) return GLINT_ERR_INVALID_ARGUMENT;
    const size_t R = b->regions.size();
    cudaSetDevice(b->device);
    for (size_t r = 0; r < R; ++r) {
        if (!d_points[r]) return GLINT_ERR_INVALID_ARGUMENT;
        if (glint::serve_only_refused(b->regions[r], "batch step")) return GLINT_ERR_STATE;
        if (!glint::device_points(b->regions[r], d_points[r])) return GLINT_ERR_INVALID_ARGUMENT;
    }
    /* the graph reads every region's step parameters from host memory when
     * it runs: the previous timestep must be done before they change */
    if (b->launched) {
        const cudaError_t e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) return batch_fail(b, e, "batch step");
    }
    /* work a caller queued on a region's own stream (a search, a flush) goes
     * first */
    for (size_t r = 0; r < R; ++r) {
        cudaEventRecord(b->pre_ev[r], b->regions[r]->stream);
        cudaStreamWaitEvent(b->stream, b->pre_ev[r], 0);
    }
    for (glint_ctx *c : b->regions) glint::begin_step(c, cur_time);
    const bool same = b->exec && std::equal(b->src.begin(), b->src.end(), d_points);
    if (!same) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return batch_fail(b, e, "batch capture");
        launch_batch_step(b, d_points);
        e = cudaStreamEndCapture(b->stream, &b->graph);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) return batch_fail(b, e, "batch capture");
        b->src.assign(d_points, d_points + R);
    }
    cudaError_t e = cudaGraphLaunch(b->exec, b->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return batch_fail(b, e, "batch step");
    b->launched = true;
    return GLINT_OK;
}

extern "C" glint_status glint_batch_sync(glint_batch *b, glint_step_stats *stats) {
    if (!b) return GLINT_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    const cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return batch_fail(b, e, "batch sync");
    glint_status first = GLINT_OK;
    for (size_t r = 0; r < b->regions.size(); ++r) {
        const glint_status st = glint_sync(b->regions[r], stats ? &stats[r] : nullptr);
        if (st != GLINT_OK && first == GLINT_OK) first = st;
    }
    return first;
}
