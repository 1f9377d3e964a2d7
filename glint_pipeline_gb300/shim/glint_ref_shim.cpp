/*
 * glint_ref_shim.cpp -- the reference's GPU seam implemented on the C ABI.
 *
 * Linked into the reference instead of cuda/geometry.cu, this file defines
 * the two functions tracing/process.cpp declares under USE_GPU
 * (tracing/process.cpp:373-376):
 *
 *   workbench *cuda_create_device_bench(workbench *bench, gpu_info *gpu);
 *   void process_with_gpu(workbench *bench, workbench *d_bench, gpu_info *gpu);
 *
 * with the reference's own types, so tracer::process and straight_dump link
 * unchanged.  It is compiled against the reference's headers (include path =
 * the reference's src/ directory) and linked with libglint.so.
 *
 * What it maps, per call of the reference's loop:
 *   configuration fields      -> glint_config (util/config.h:15-114), with
 *                                the flush inside the step once more than
 *                                kv_restriction keys are pending, as
 *                                cuda/geometry.cu:1752 does
 *   bench->mbr, bench->schema -> glint_box, glint_schema_init (QTSchema layout)
 *   bench->points, cur_time   -> glint_step
 *   glint_step_stats          -> grid_check_counter, filter_list_index,
 *                                num_taken_buckets, num_active_meetings, pro.*_time
 *   search_single / search_multi (+ search_single_pid, search_multi_pid[],
 *   search_multi_length)      -> glint_active_search into search_single_list /
 *                                single_find_count and search_multi_list /
 *                                multi_find_count (cuda/geometry.cu:605-663)
 *   a flush                   -> h_keys[offset] (packed CTF keys),
 *                                h_oversize_buffers[offset], h_sids[offset],
 *                                h_CTF_capacity[offset], h_ctfs[offset],
 *                                h_bitmaps[offset], h_bitmap_mbrs[offset] and
 *                                MemTable_count++ (cuda/geometry.cu:1757-1762,
 *                                1795-1827, 2020-2035, 2129), which
 *                                straight_dump reads (tracing/process.cpp:254-348)
 *   identified meetings       -> h_meetings_ps[0..h_meetings_count) when the
 *                                caller allocated it (the CPU path's buffer;
 *                                the reference's GPU path keeps them on the device)
 * Errors follow the reference's convention (CUDA_SAFE_CALL exits,
 * cuda/cuda_util.cuh:19-27): a failing call prints and exits.
 */
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tracing/workbench.h"
#include "cuda/mygpu.h"

#include "glint.h"

namespace {

glint_ctx *g_ctx = nullptr;
std::vector<glint_meeting> g_meet;
std::vector<glint_search_info> g_found;
std::vector<glint_ctf_meta> g_ctfs;
uint64_t g_key_capacity = 0;   /* keys each h_keys[i] holds */
/* the device workbench's start_time_min/max, which process_with_gpu folds
 * into the host's at every flush and resets after it (cuda/geometry.cu:
 * 1755-1756, 2096-2097) */
uint32_t g_dev_start_min = 0, g_dev_start_max = 0;

void check(glint_status st, const char *what) {
    if (st == GLINT_OK) return;
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, glint_status_string(st), glint_last_error(g_ctx));
    std::exit(EXIT_FAILURE);
}

void fail(const char *what) {
    std::fprintf(stderr, "%s\n", what);
    std::exit(EXIT_FAILURE);
}

/* the active multi-search over `pids`, into list[0..cap); returns the count */
uint32_t search_into(const uint32_t *pids, uint32_t npids, search_info_unit *list, uint32_t cap, bool with_pid) {
    uint64_t n = 0;
    check(glint_active_search(g_ctx, pids, npids, nullptr, 0, &n), "glint_active_search");
    g_found.resize(n);
    if (n) check(glint_active_search(g_ctx, pids, npids, g_found.data(), n, &n), "glint_active_search");
    if (n > cap) fail("active search: more records than search_*_capacity (the reference asserts)");
    for (uint64_t i = 0; i < n; ++i) {
        search_info_unit &u = list[i];
        if (with_pid) u.pid = g_found[i].pid;
        u.target = g_found[i].target;
        u.start = g_found[i].start;
        u.end = g_found[i].end;
        u.low0 = g_found[i].mbr[0];
        u.low1 = g_found[i].mbr[1];
        u.high0 = g_found[i].mbr[2];
        u.high1 = g_found[i].mbr[3];
    }
    return (uint32_t)n;
}

/* the flushed block into the host buffers straight_dump reads */
void hand_over_flush(workbench *bench) {
    const configuration *c = bench->config;
    uint32_t offset = (bench->ctb_count % 2 == 1) ? c->MemTable_capacity / 2 : 0;
    offset += bench->MemTable_count;
    if (offset >= c->MemTable_capacity) fail("flush with every MemTable taken (the caller did not dump)");
    glint_store_info info;
    check(glint_store_read(g_ctx, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &info),
          "glint_store_read");
    if (info.key_bytes > g_key_capacity * sizeof(__uint128_t)) fail("flushed keys exceed h_keys");
    if (info.oversize_kv_count > c->oversize_buffer_capacity)
        fail("oversize keys exceed oversize_buffer_capacity (the reference asserts)");
    oversize_buffer &ob = bench->h_oversize_buffers[offset];
    g_ctfs.resize(c->CTF_count);
    static_assert(sizeof(f_box) == 4 * sizeof(float), "f_box layout");
    check(glint_store_read(g_ctx, reinterpret_cast<uint8_t *>(bench->h_keys[offset]), bench->h_sids[offset],
                           bench->h_CTF_capacity[offset], g_ctfs.data(), bench->h_bitmaps[offset], ob.keys,
                           reinterpret_cast<float *>(ob.boxes), ob.o_bitmaps, &info),
          "glint_store_read");
    /* the rest of h_keys[offset]: the reference copies kv_count 16-byte words
     * of its zero-initialised packed buffer */
    const uint64_t copied = std::min<uint64_t>(info.kv_count, g_key_capacity) * sizeof(__uint128_t);
    if (copied > info.key_bytes)
        std::memset(reinterpret_cast<uint8_t *>(bench->h_keys[offset]) + info.key_bytes, 0, copied - info.key_bytes);
    ob.oversize_kv_count = info.oversize_kv_count;
    ob.start_time_min = info.oversize_start_time_min;
    ob.start_time_max = info.oversize_start_time_max;
    ob.end_time_min = info.oversize_end_time_min;
    ob.end_time_max = info.oversize_end_time_max;
    for (uint32_t i = 0; i < c->CTF_count; ++i) {
        CTF &f = bench->h_ctfs[offset][i];
        const glint_ctf_meta &m = g_ctfs[i];
        f.ctf_mbr.low[0] = m.ctf_mbr[0];
        f.ctf_mbr.low[1] = m.ctf_mbr[1];
        f.ctf_mbr.high[0] = m.ctf_mbr[2];
        f.ctf_mbr.high[1] = m.ctf_mbr[3];
        f.keys = nullptr;
        f.bitmap = nullptr;
        f.CTF_kv_capacity = m.CTF_kv_capacity;
        f.start_time_min = m.start_time_min;
        f.start_time_max = m.start_time_max;
        f.end_time_min = m.end_time_min;
        f.end_time_max = m.end_time_max;
        f.ctf_bitmap_size = m.ctf_bitmap_size;
        f.key_bit = m.key_bit;
        f.id_bit = m.id_bit;
        f.duration_bit = m.duration_bit;
        f.end_bit = m.end_bit;
        f.low_x_bit = m.low_x_bit;
        f.low_y_bit = m.low_y_bit;
        f.edge_bit = m.edge_bit;
        f.mbr_bit = m.mbr_bit;
        f.x_grid = m.x_grid;
        f.y_grid = m.y_grid;
    }
    /* d_bitmap_mbrs is never written by the flush kernels: zeros */
    std::memset(bench->h_bitmap_mbrs[offset], 0, sizeof(box) * c->CTF_count);
    bench->start_time_min = std::min(bench->start_time_min, g_dev_start_min);
    bench->start_time_max = std::max(bench->start_time_max, g_dev_start_max);
    g_dev_start_min = 0xffffffffu;
    g_dev_start_max = 0;
    bench->MemTable_count++;
}

} // namespace

workbench *cuda_create_device_bench(workbench *bench, gpu_info *gpu) {
    const configuration *c = bench->config;
    glint_config cfg;
    glint_config_defaults(&cfg, c->num_objects);
    cfg.grid_capacity = c->grid_capacity;
    cfg.grid_amplify = c->grid_amplify;
    cfg.num_meeting_buckets = c->num_meeting_buckets;
    cfg.reach_distance = c->reach_distance;
    cfg.min_meet_time = c->min_meet_time;
    cfg.max_meet_time = c->max_meet_time;
    cfg.schema_update_delay = c->schema_update_delay;
    cfg.dynamic_schema = c->dynamic_schema;
    cfg.phased_lookup = c->phased_lookup;
    cfg.start_time = c->start_time;
    cfg.x_buffer = c->x_buffer;
    cfg.y_buffer = c->y_buffer;
    cfg.G_bytes = c->G_bytes;
    cfg.CTF_count = c->CTF_count;
    cfg.split_num = c->split_num;
    cfg.dProbFalse = bench->dProbFalse;
    cfg.auto_flush = 1;
    cfg.kv_restriction = c->kv_restriction;
    /* the reference's kv_capacity adds 1e6 keys, which one step of a large
     * population can exceed; the context keeps its own larger default and
     * the host buffers are sized to it */
    cfg.kv_capacity = 0;
    cfg.device = gpu ? (uint32_t)gpu->device_id : 0u;
    glint_box mbr;
    mbr.low[0] = bench->mbr.low[0];
    mbr.low[1] = bench->mbr.low[1];
    mbr.high[0] = bench->mbr.high[0];
    mbr.high[1] = bench->mbr.high[1];
    /* the schema partitioner::build_schema left on the host (QTSchema layout) */
    static_assert(sizeof(QTSchema) == sizeof(glint_schema_node), "QTSchema layout");
    glint_schema_init init = {};
    init.nodes = reinterpret_cast<const glint_schema_node *>(bench->schema);
    init.num_nodes = bench->schema_stack_capacity;
    init.schema_stack_index = bench->schema_stack_index;
    init.grids_stack_index = bench->grids_stack_index;
    init.schema_stack = bench->schema_stack;
    init.grids_stack = bench->grids_stack;
    check(glint_create(&cfg, &mbr, nullptr, &init, &g_ctx), "glint_create");
    /* page-locked key buffers of the MemTables (cuda/geometry.cu:1462-1463) */
    const uint64_t restriction = c->kv_restriction;
    g_key_capacity = std::max<uint64_t>(c->kv_capacity,
                                        restriction + std::max<uint64_t>(1000000ull, 4ull * c->num_objects));
    for (uint32_t i = 0; i < c->MemTable_capacity; ++i) {
        void *p = nullptr;
        check(glint_host_alloc(g_key_capacity * sizeof(__uint128_t), &p), "glint_host_alloc");
        std::memset(p, 0, g_key_capacity * sizeof(__uint128_t));
        bench->h_keys[i] = static_cast<__uint128_t *>(p);
    }
    g_dev_start_min = bench->start_time_min;
    g_dev_start_max = bench->start_time_max;
    /* the device-side workbench handle is the context; the caller only passes it back */
    return bench;
}

void process_with_gpu(workbench *bench, workbench *d_bench, gpu_info *gpu) {
    (void)d_bench;
    (void)gpu;
    glint_step_stats st;
    check(glint_step(g_ctx, reinterpret_cast<const double *>(bench->points), bench->cur_time, &st), "glint_step");
    bench->grid_check_counter = st.checks;
    bench->filter_list_index = st.border_objects;
    bench->num_taken_buckets = st.num_taken_buckets;
    bench->num_active_meetings = st.num_active_meetings;
    bench->pro.copy_time += st.ms[0];
    bench->pro.partition_time += st.ms[1];
    bench->pro.filter_time += st.ms[2];
    bench->pro.refine_time += st.ms[3] + st.ms[4];
    bench->pro.meeting_identify_time += st.ms[5];
    bench->pro.index_update_time += st.ms[6];
    bench->pro.cuda_sort_time += st.flush_ms;
    /* the active searches of cuda_identify_meetings, over the table as this
     * step left it; records come in bucket order */
    if (bench->search_single) {
        bench->single_find_count = search_into(&bench->search_single_pid, 1, bench->search_single_list,
                                               bench->config->search_single_capacity, false);
    }
    if (bench->search_multi) {
        bench->multi_find_count = search_into(bench->search_multi_pid, bench->search_multi_length,
                                              bench->search_multi_list, bench->config->search_multi_capacity, true);
    }
    if (st.flushed) hand_over_flush(bench);
    if (bench->h_meetings_ps) {
        uint64_t n = 0;
        check(glint_meetings(g_ctx, nullptr, 0, &n), "glint_meetings");
        g_meet.resize(n);
        if (n) check(glint_meetings(g_ctx, g_meet.data(), n, &n), "glint_meetings");
        const uint64_t cap = (uint64_t)bench->config->num_objects * 10;  /* h_meetings_ps, workbench.cpp:167 */
        const uint64_t m = std::min<uint64_t>(n, cap);
        for (uint64_t i = 0; i < m; ++i) {
            meeting_unit &u = bench->h_meetings_ps[i];
            u.key = cantorPairing(g_meet[i].pid1, g_meet[i].pid2);
            u.start = g_meet[i].start;
            u.end = g_meet[i].end;
            u.mbr.low[0] = g_meet[i].mbr[0];
            u.mbr.low[1] = g_meet[i].mbr[1];
            u.mbr.high[0] = g_meet[i].mbr[2];
            u.mbr.high[1] = g_meet[i].mbr[3];
        }
        bench->h_meetings_count = (uint)n;
    }
}
