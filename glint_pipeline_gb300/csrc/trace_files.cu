/*
 * trace_files.cu -- the reference's trace chunk files, read ahead on a host
 * thread.
 *
 * The reference stores a trace as files <trace_path><st>_<num_objects>.tr,
 * each holding 100 steps of num_objects Points (two doubles, lon then lat),
 * step after step, with no header (tools/datagen.cpp:18-26); tracer::loadData
 * reads one whole file before the 100 steps it covers
 * (tracing/process.cpp:128-144).  Here a reader thread fills a ring of
 * page-locked step buffers a few steps ahead of the caller, so that file
 * reads overlap with the device steps and the buffers can feed
 * glint_pipe_submit directly.
 */
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "glint.h"

namespace {

constexpr uint32_t kChunkSteps = 100; /* steps per file, tools/datagen.cpp:22 */

std::string chunk_path(const std::string &prefix, uint32_t st, uint32_t n) {
    return prefix + std::to_string(st) + "_" + std::to_string(n) + ".tr";
}

thread_local std::string g_trace_error;

} // namespace

struct glint_trace {
    std::string prefix;
    uint32_t n = 0, first = 0, steps = 0, ring = 0;
    size_t step_bytes = 0;
    std::vector<double *> buf;
    std::vector<bool> pinned;
    std::vector<int64_t> held;     /* step in each ring slot, -1 when empty */
    std::mutex mu;
    std::condition_variable cv;
    int64_t next_read = 0;         /* next step the reader loads */
    int64_t released = -1;         /* steps up to this one may be overwritten */
    bool stop = false;
    std::string error;
    std::thread reader;
};

static void trace_reader(glint_trace *tr) {
    FILE *f = nullptr;
    uint32_t open_chunk = ~0u;
    for (;;) {
        int64_t s;
        uint32_t slot;
        {
            std::unique_lock<std::mutex> lk(tr->mu);
            tr->cv.wait(lk, [&] {
                return tr->stop || (tr->next_read < (int64_t)tr->steps &&
                                    tr->next_read - (int64_t)tr->ring <= tr->released);
            });
            if (tr->stop || tr->next_read >= (int64_t)tr->steps) break;
            s = tr->next_read;
            slot = (uint32_t)(s % tr->ring);
        }
        const uint32_t t = tr->first + (uint32_t)s;
        const uint32_t chunk = t / kChunkSteps * kChunkSteps;
        std::string err;
        if (chunk != open_chunk) {
            if (f) fclose(f);
            f = fopen(chunk_path(tr->prefix, chunk, tr->n).c_str(), "rb");
            open_chunk = chunk;
            if (!f) err = "cannot open " + chunk_path(tr->prefix, chunk, tr->n);
        }
        if (err.empty()) {
            const long off = (long)((t - chunk) * tr->step_bytes);
            if (fseek(f, off, SEEK_SET) != 0 || fread(tr->buf[slot], 1, tr->step_bytes, f) != tr->step_bytes)
                err = "short file " + chunk_path(tr->prefix, chunk, tr->n) + " at step " + std::to_string(t);
        }
        std::lock_guard<std::mutex> lk(tr->mu);
        if (!err.empty()) {
            tr->error = err;
            tr->stop = true;
            tr->cv.notify_all();
            break;
        }
        tr->held[slot] = s;
        tr->next_read = s + 1;
        tr->cv.notify_all();
    }
    if (f) fclose(f);
}

static void trace_free(glint_trace *tr) {
    for (size_t k = 0; k < tr->buf.size(); ++k) {
        if (!tr->buf[k]) continue;
        if (tr->pinned[k]) cudaFreeHost(tr->buf[k]);
        else std::free(tr->buf[k]);
    }
}

extern "C" glint_status glint_trace_open(const char *prefix, uint32_t num_objects, uint32_t first_step,
                                         uint32_t num_steps, uint32_t ring, glint_trace **out) {
    if (!prefix || !out || num_objects == 0 || ring < 3) {
        g_trace_error = "trace open: invalid argument (the ring needs at least 3 steps)";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    glint_trace *tr = new glint_trace();
    tr->prefix = prefix;
    tr->n = num_objects;
    tr->first = first_step;
    tr->steps = num_steps;
    tr->ring = ring;
    tr->step_bytes = (size_t)num_objects * 2 * sizeof(double);
    tr->buf.assign(ring, nullptr);
    tr->pinned.assign(ring, false);
    tr->held.assign(ring, -1);
    for (uint32_t k = 0; k < ring; ++k) {
        void *p = nullptr;
        if (cudaMallocHost(&p, tr->step_bytes) == cudaSuccess) {
            tr->pinned[k] = true;
        } else {
            cudaGetLastError();
            p = std::malloc(tr->step_bytes); /* no device: ordinary memory */
        }
        if (!p) {
            trace_free(tr);
            delete tr;
            g_trace_error = "trace open: out of host memory";
            return GLINT_ERR_OUT_OF_MEMORY;
        }
        tr->buf[k] = (double *)p;
    }
    tr->reader = std::thread(trace_reader, tr);
    *out = tr;
    return GLINT_OK;
}

extern "C" glint_status glint_trace_step(glint_trace *tr, uint32_t t, const double **points) {
    if (!tr || !points || t < tr->first || t - tr->first >= tr->steps) {
        g_trace_error = "trace step: outside the opened range";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    const int64_t s = (int64_t)(t - tr->first);
    std::unique_lock<std::mutex> lk(tr->mu);
    /* the two most recent steps handed out stay valid: the last one may still
     * be in an asynchronous copy */
    if (s - 2 > tr->released) {
        tr->released = s - 2;
        tr->cv.notify_all();
    }
    const uint32_t slot = (uint32_t)(s % tr->ring);
    tr->cv.wait(lk, [&] { return tr->held[slot] == s || !tr->error.empty() || s < tr->next_read - (int64_t)tr->ring; });
    if (tr->held[slot] != s) {
        g_trace_error = tr->error.empty() ? "trace step: that step has left the ring" : "trace: " + tr->error;
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    *points = tr->buf[slot];
    return GLINT_OK;
}

extern "C" glint_status glint_trace_close(glint_trace *tr) {
    if (!tr) return GLINT_OK;
    {
        std::lock_guard<std::mutex> lk(tr->mu);
        tr->stop = true;
        tr->cv.notify_all();
    }
    if (tr->reader.joinable()) tr->reader.join();
    trace_free(tr);
    delete tr;
    return GLINT_OK;
}

extern "C" const char *glint_trace_error(void) { return g_trace_error.c_str(); }

extern "C" glint_status glint_trace_write(const char *prefix, uint32_t num_objects, uint32_t first_step,
                                          const double *points, uint32_t num_steps) {
    if (!prefix || (num_steps && !points) || num_objects == 0) {
        g_trace_error = "trace write: invalid argument";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    const size_t step_bytes = (size_t)num_objects * 2 * sizeof(double);
    FILE *f = nullptr;
    uint32_t open_chunk = ~0u;
    for (uint32_t s = 0; s < num_steps; ++s) {
        const uint32_t t = first_step + s;
        const uint32_t chunk = t / kChunkSteps * kChunkSteps;
        if (chunk != open_chunk) {
            if (f) fclose(f);
            const std::string path = chunk_path(prefix, chunk, num_objects);
            /* a file continued at a later step keeps its earlier steps */
            f = fopen(path.c_str(), t == chunk ? "wb" : "r+b");
            if (!f) f = fopen(path.c_str(), "wb");
            open_chunk = chunk;
            if (!f) {
                g_trace_error = "trace write: cannot create " + path;
                return GLINT_ERR_INVALID_ARGUMENT;
            }
        }
        if (fseek(f, (long)((t - chunk) * step_bytes), SEEK_SET) != 0 ||
            fwrite(points + (size_t)s * num_objects * 2, 1, step_bytes, f) != step_bytes) {
            fclose(f);
            g_trace_error = "trace write: short write";
            return GLINT_ERR_INVALID_ARGUMENT;
        }
    }
    if (f) fclose(f);
    return GLINT_OK;
}
