/*
 * glint_pipe.cu -- pipelined stepping from host memory.
 *
 * The reference copies each step's points to the device and its results back
 * inside process_with_gpu, one after the other (cuda/geometry.cu:1625,
 * 2142-2157).  Here the copy of step t+1's points runs on a copy stream into
 * the second of two device buffers while step t computes.  At the end of
 * each step a kernel gathers its meetings from the device log into one of two
 * device staging buffers; once the host knows the count, the copy engine
 * brings them into one of two page-locked result buffers while the next step
 * runs.  (Kernel writes straight into mapped host memory were measured at
 * about 26 GB/s, the copy engine at about 190 GB/s.)
 *
 * Order of one glint_pipe_submit(t + 1):
 *   1. copy stream: wait until the step that last read input buffer
 *      (t + 1) % 2 is done, copy the points into it, record `copied`;
 *   2. finish step t (glint_sync: its statistics, and the automatic flush,
 *      which therefore still falls between step t and step t + 1 as in the
 *      reference); copy stream: step t's meetings to the host, record
 *      `fetched`;
 *   3. main stream: wait for `copied`, enqueue step t + 1 on that buffer,
 *      then the gathering of its meetings into staging buffer (t + 1) % 2.
 * Results of a step stay valid until the submit two steps later.
 */
#include <cstring>

#include "glint_internal.cuh"

namespace {

__global__ void __launch_bounds__(256) k_gather_meetings(const glint_meeting *__restrict__ log, uint64_t log_cap,
                                                          const glint::DevCounters *__restrict__ cnt,
                                                          glint_meeting *__restrict__ out, uint64_t cap) {
    const unsigned long long n = cnt->meetings;
    const unsigned long long begin = cnt->log_step_begin;
    const unsigned long long m = n < cap ? n : cap;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < m;
         i += (unsigned long long)gridDim.x * blockDim.x)
        out[i] = log[(begin + i) % log_cap];
}

} // namespace

struct glint_pipe {
    glint_ctx *ctx = nullptr;
    uint64_t cap = 0;                      /* meetings per result buffer */
    double *d_in[2] = {nullptr, nullptr};  /* device input buffers */
    glint_meeting *d_stage[2] = {nullptr, nullptr}; /* a step's meetings, gathered on the device */
    glint_meeting *h_out[2] = {nullptr, nullptr};   /* page-locked */
    uint64_t count[2] = {0, 0};
    cudaStream_t copy = nullptr;           /* points in */
    cudaStream_t fetch = nullptr;          /* meetings out */
    cudaEvent_t copied[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    cudaEvent_t fetched[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    /* the step in flight and the last finished one */
    bool pending = false;
    uint32_t pending_time = 0, pending_slot = 0;
    bool have_last = false;
    uint32_t last_time = 0, last_slot = 0;
    glint_step_stats last_stats;
};

static void pipe_release(glint_pipe *p) {
    for (int k = 0; k < 2; ++k) {
        if (p->d_in[k]) cudaFree(p->d_in[k]);
        if (p->d_stage[k]) cudaFree(p->d_stage[k]);
        if (p->h_out[k]) cudaFreeHost(p->h_out[k]);
        if (p->copied[k]) cudaEventDestroy(p->copied[k]);
        if (p->done[k]) cudaEventDestroy(p->done[k]);
        if (p->fetched[k]) cudaEventDestroy(p->fetched[k]);
    }
    if (p->copy) cudaStreamDestroy(p->copy);
    if (p->fetch) cudaStreamDestroy(p->fetch);
}

/* finishes the step in flight (statistics, automatic flush) and starts the
 * copy of its meetings to the host */
static glint_status pipe_finish(glint_pipe *p) {
    if (!p->pending) return GLINT_OK;
    p->pending = false;
    const glint_status st = glint_sync(p->ctx, &p->last_stats);
    p->have_last = true;
    p->last_time = p->pending_time;
    p->last_slot = p->pending_slot;
    const uint32_t k = p->last_slot;
    p->count[k] = p->last_stats.meetings;
    const uint64_t m = p->count[k] < p->cap ? p->count[k] : p->cap;
    cudaError_t e = cudaSuccess;
    if (m) e = cudaMemcpyAsync(p->h_out[k], p->d_stage[k], sizeof(glint_meeting) * m, cudaMemcpyDeviceToHost, p->fetch);
    if (e == cudaSuccess) e = cudaEventRecord(p->fetched[k], p->fetch);
    if (e != cudaSuccess) {
        p->ctx->last_error = std::string("pipe fetch: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    return st;
}

extern "C" glint_status glint_pipe_create(glint_ctx *c, uint64_t result_capacity, glint_pipe **out) {
    if (!c || !out) return GLINT_ERR_INVALID_ARGUMENT;
    if (glint::serve_only_refused(c, "pipe")) return GLINT_ERR_STATE;
    *out = nullptr;
    cudaSetDevice(c->device);
    glint_pipe *p = new glint_pipe();
    p->ctx = c;
    p->cap = result_capacity ? result_capacity : (uint64_t)c->N;
    std::memset(&p->last_stats, 0, sizeof(p->last_stats));
    cudaError_t e = cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->fetch, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaMalloc((void **)&p->d_in[k], sizeof(double2) * (size_t)(c->N ? c->N : 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&p->d_stage[k], sizeof(glint_meeting) * (p->cap ? p->cap : 1));
        if (e == cudaSuccess) e = cudaMallocHost((void **)&p->h_out[k], sizeof(glint_meeting) * (p->cap ? p->cap : 1));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->copied[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->done[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fetched[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        pipe_release(p);
        delete p;
        c->last_error = std::string("pipe: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    *out = p;
    return GLINT_OK;
}

extern "C" glint_status glint_pipe_destroy(glint_pipe *p) {
    if (!p) return GLINT_OK;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
    cudaStreamSynchronize(p->copy);
    cudaStreamSynchronize(p->fetch);
    pipe_release(p);
    delete p;
    return GLINT_OK;
}

extern "C" glint_status glint_pipe_submit(glint_pipe *p, const double *points, uint32_t cur_time) {
    if (!p || !points) return GLINT_ERR_INVALID_ARGUMENT;
    glint_ctx *c = p->ctx;
    cudaSetDevice(c->device);
    /* the slot after the step in flight (or after the last one) */
    const uint32_t slot = p->pending ? (p->pending_slot ^ 1u) : (p->have_last ? (p->last_slot ^ 1u) : 0u);
    /* 1. the copy, behind the step that last read this buffer */
    if (p->used[slot]) cudaStreamWaitEvent(p->copy, p->done[slot], 0);
    cudaError_t e = cudaMemcpyAsync(p->d_in[slot], points, sizeof(double2) * (size_t)c->N, cudaMemcpyHostToDevice,
                                    p->copy);
    if (e == cudaSuccess) e = cudaEventRecord(p->copied[slot], p->copy);
    if (e != cudaSuccess) {
        c->last_error = std::string("pipe copy: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    /* 2. the step in flight ends (and flushes) before this one starts */
    const glint_status fs = pipe_finish(p);
    if (fs != GLINT_OK) return fs;
    /* 3. the step and the export of its meetings */
    cudaStreamWaitEvent(c->stream, p->copied[slot], 0);
    const glint_status st = glint::enqueue_device_step_plain(c, p->d_in[slot], cur_time);
    if (st != GLINT_OK) return st;
    /* the staging buffer is free once its last copy to the host is done */
    if (p->used[slot]) cudaStreamWaitEvent(c->stream, p->fetched[slot], 0);
    k_gather_meetings<<<152 * 4, 256, 0, c->stream>>>(c->d_log, c->log_cap, c->d_cnt, p->d_stage[slot], p->cap);
    e = cudaEventRecord(p->done[slot], c->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        c->last_error = std::string("pipe step: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    p->used[slot] = true;
    p->pending = true;
    p->pending_time = cur_time;
    p->pending_slot = slot;
    return GLINT_OK;
}

extern "C" glint_status glint_pipe_result(glint_pipe *p, uint32_t cur_time, glint_step_stats *stats,
                                          const glint_meeting **meetings, uint64_t *n) {
    if (!p) return GLINT_ERR_INVALID_ARGUMENT;
    glint_ctx *c = p->ctx;
    cudaSetDevice(c->device);
    if (p->pending && p->pending_time == cur_time) {
        const glint_status st = pipe_finish(p);
        if (st != GLINT_OK) return st;
    }
    if (!p->have_last || p->last_time != cur_time) {
        c->last_error = "pipe result: that step is not the last finished one";
        return GLINT_ERR_STATE;
    }
    cudaError_t e = cudaEventSynchronize(p->fetched[p->last_slot]);
    if (e != cudaSuccess) {
        c->last_error = std::string("pipe result: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    const uint64_t total = p->count[p->last_slot];
    if (stats) *stats = p->last_stats;
    if (meetings) *meetings = p->h_out[p->last_slot];
    if (n) *n = total;
    if (total > p->cap) {
        c->last_error = "pipe result: more meetings than the result capacity (read them with glint_meetings)";
        return GLINT_ERR_CAPACITY;
    }
    return GLINT_OK;
}
