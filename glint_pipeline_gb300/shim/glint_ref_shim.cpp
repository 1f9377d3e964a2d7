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
 * with the reference's own types, so tracer::process links unchanged.  It is
 * compiled against the reference's headers (include path = the reference's
 * src/ directory) and linked with libglint.so.
 *
 * What it maps:
 *   configuration fields      -> glint_config   (util/config.h:15-114)
 *   bench->mbr, bench->schema -> glint_box, glint_schema_init (QTSchema layout)
 *   bench->points, cur_time   -> glint_step
 *   glint_step_stats          -> grid_check_counter, filter_list_index,
 *                                num_taken_buckets, num_active_meetings, pro.*_time
 *   identified meetings       -> batch_meet() into h_meetings_ps, as
 *                                update_meetings does (tracing/meeting.cpp:11-24)
 * Errors follow the reference's convention (CUDA_SAFE_CALL exits,
 * cuda/cuda_util.cuh:19-27): a failing call prints and exits.
 */
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tracing/workbench.h"
#include "cuda/mygpu.h"

#include "glint.h"

namespace {

glint_ctx *g_ctx = nullptr;
std::vector<glint_meeting> g_meet;
std::vector<meeting_unit> g_units;

void check(glint_status st, const char *what) {
    if (st == GLINT_OK) return;
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, glint_status_string(st), glint_last_error(g_ctx));
    std::exit(EXIT_FAILURE);
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
    cfg.x_buffer = c->x_buffer;
    cfg.y_buffer = c->y_buffer;
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
    uint64_t n = 0;
    check(glint_meetings(g_ctx, nullptr, 0, &n), "glint_meetings");
    g_meet.resize(n);
    if (n) check(glint_meetings(g_ctx, g_meet.data(), n, &n), "glint_meetings");
    g_units.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
        meeting_unit &u = g_units[i];
        u.key = cantorPairing(g_meet[i].pid1, g_meet[i].pid2);
        u.start = g_meet[i].start;
        u.end = g_meet[i].end;
        u.mbr.low[0] = g_meet[i].mbr[0];
        u.mbr.low[1] = g_meet[i].mbr[1];
        u.mbr.high[0] = g_meet[i].mbr[2];
        u.mbr.high[1] = g_meet[i].mbr[3];
    }
    bench->batch_meet(g_units.data(), (uint)n);
}
