/*
 * glint_batch.cu -- the batching form: many independent regions advanced
 * together on one GPU.
 *
 * Each region is a context of its own (its schema, meeting table, store) with
 * its own CUDA stream; its step is captured once as a CUDA graph
 * (glint_config.use_graph) and replayed every timestep from the region's
 * fixed device input buffer.  glint_batch_step launches every region's graph
 * before waiting for any, so the kernels of small regions, which alone would
 * leave most of the GPU idle, run side by side with those of large ones.  The
 * reference runs one region per process (tracing/process.cpp:401-462).
 */
#include <cstring>
#include <vector>

#include "glint_internal.cuh"

struct glint_batch {
    std::vector<glint_ctx *> regions;
};

extern "C" glint_status glint_batch_create(uint32_t n, const glint_config *cfgs, const glint_box *mbrs,
                                           const double *const *first_points, glint_batch **out) {
    if (!out || n == 0 || !cfgs || !mbrs || !first_points) return GLINT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    glint_batch *b = new glint_batch();
    for (uint32_t r = 0; r < n; ++r) {
        glint_config cfg = cfgs[r];
        cfg.use_graph = 1;
        cfg.timing = 0;
        glint_ctx *c = nullptr;
        const glint_status st = glint_create(&cfg, &mbrs[r], first_points[r], nullptr, &c);
        if (st != GLINT_OK) {
            for (glint_ctx *x : b->regions) glint_destroy(x);
            delete b;
            return st;
        }
        b->regions.push_back(c);
    }
    *out = b;
    return GLINT_OK;
}

extern "C" glint_status glint_batch_destroy(glint_batch *b) {
    if (!b) return GLINT_OK;
    for (glint_ctx *c : b->regions) glint_destroy(c);
    delete b;
    return GLINT_OK;
}

extern "C" uint32_t glint_batch_regions(const glint_batch *b) { return b ? (uint32_t)b->regions.size() : 0u; }

extern "C" glint_ctx *glint_batch_region(glint_batch *b, uint32_t r) {
    return (b && r < b->regions.size()) ? b->regions[r] : nullptr;
}

extern "C" glint_status glint_batch_step(glint_batch *b, const double *const *d_points, uint32_t cur_time) {
    if (!b || !d_points) return GLINT_ERR_INVALID_ARGUMENT;
    for (size_t r = 0; r < b->regions.size(); ++r) {
        const glint_status st = glint_step_device(b->regions[r], d_points[r], cur_time);
        if (st != GLINT_OK) return st;
    }
    return GLINT_OK;
}

extern "C" glint_status glint_batch_sync(glint_batch *b, glint_step_stats *stats) {
    if (!b) return GLINT_ERR_INVALID_ARGUMENT;
    glint_status first = GLINT_OK;
    for (size_t r = 0; r < b->regions.size(); ++r) {
        const glint_status st = glint_sync(b->regions[r], stats ? &stats[r] : nullptr);
        if (st != GLINT_OK && first == GLINT_OK) first = st;
    }
    return first;
}
