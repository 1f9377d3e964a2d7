/*
 * ref_driver.cpp -- per-step driver around the reference's own CPU stages.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/build_ref.sh) together with
 * the unmodified reference sources tracing/{filter,refinement,meeting,
 * workbench,step_merge,analyze}.cpp into oracle/_ref/libglintref.so, so that
 * golden fixtures and the CPU baseline come from the reference's code itself.
 * Nothing in the product links or loads this.
 *
 * The per-step sequence mirrors the CPU branch of tracer::process()
 * (tracing/process.cpp:431-612): reset(), points = trace + t*N, cur_time,
 * filter(), reachability(), update_meetings(), then update_schema() when the
 * schema is dynamic.  The schema is built once from the first step's points
 * with partitioner::build_schema (tracing/filter.cpp:27-93), as
 * tracing/process.cpp:401-404 does.
 */
#include "tracing/partitioner.h"
#include "tracing/workbench.h"

#include <cstdint>
#include <cstring>

extern "C" {

struct ref_config {
    uint32_t num_objects;
    uint32_t num_threads;
    uint32_t grid_capacity;
    uint32_t schema_update_delay;
    uint32_t min_meet_time;
    uint32_t dynamic_schema;
    uint64_t num_meeting_buckets;
    double grid_amplify;
    double reach_distance;
    uint32_t start_time;
    uint32_t pad;
};

struct ref_handle {
    configuration *config;
    partitioner *part;
    workbench *bench;
    Point *points;      /* copy of the current step's points */
    double ms_filter, ms_refine, ms_meet, ms_schema;
    uint32_t checks;     /* grid_check_counter right after reachability() */
};

struct ref_counts {
    uint32_t grid_check_counter;
    uint32_t kv_count;
    uint64_t num_taken_buckets;
    uint32_t num_active_meetings;
    uint32_t grids_stack_index;
    uint32_t schema_stack_index;
    uint32_t grids_stack_capacity;
    uint32_t schema_stack_capacity;
    uint32_t grid_capacity;
    double x_buffer;
    double y_buffer;
    double ms_filter, ms_refine, ms_meet, ms_schema;
};

void *ref_create(const ref_config *rc, const double *mbr4, const double *points_xy) {
    ref_handle *h = new ref_handle();
    configuration *c = new configuration();
    c->num_objects = rc->num_objects;
    c->num_threads = rc->num_threads ? rc->num_threads : 1;
    c->grid_capacity = rc->grid_capacity;
    c->zone_capacity = rc->grid_capacity;
    c->schema_update_delay = rc->schema_update_delay;
    c->min_meet_time = rc->min_meet_time;
    c->dynamic_schema = rc->dynamic_schema != 0;
    c->num_meeting_buckets = rc->num_meeting_buckets;
    c->grid_amplify = rc->grid_amplify;
    c->reach_distance = rc->reach_distance;
    c->start_time = rc->start_time;
    c->gpu = false;
    c->phased_lookup = true;
    h->config = c;
    box b(mbr4[0], mbr4[1], mbr4[2], mbr4[3]);
    h->part = new partitioner(b, c);
    h->points = new Point[rc->num_objects];
    memcpy((void *)h->points, points_xy, sizeof(Point) * (size_t)rc->num_objects);
    h->bench = h->part->build_schema(h->points, rc->num_objects);
    h->bench->mbr = b;
    h->ms_filter = h->ms_refine = h->ms_meet = h->ms_schema = 0;
    h->checks = 0;
    return h;
}

/* one timestep with the reference's CPU stages; points_xy is N (x,y) pairs */
int ref_step(void *hv, const double *points_xy, uint32_t cur_time) {
    ref_handle *h = (ref_handle *)hv;
    workbench *bench = h->bench;
    memcpy((void *)h->points, points_xy, sizeof(Point) * (size_t)h->config->num_objects);
    bench->reset();
    bench->points = h->points;
    bench->cur_time = cur_time;
    struct timeval ct = get_cur_time();
    bench->filter();
    h->ms_filter = get_time_elapsed(ct, true);
    bench->reachability();
    h->ms_refine = get_time_elapsed(ct, true);
    h->checks = bench->grid_check_counter;
    bench->update_meetings();
    h->ms_meet = get_time_elapsed(ct, true);
    h->ms_schema = 0;
    if (h->config->dynamic_schema) {
        bench->update_schema();
        h->ms_schema = get_time_elapsed(ct, true);
    }
    return 0;
}

void ref_get_counts(void *hv, ref_counts *out) {
    ref_handle *h = (ref_handle *)hv;
    workbench *b = h->bench;
    out->grid_check_counter = h->checks;
    out->kv_count = b->kv_count;
    out->num_taken_buckets = b->num_taken_buckets;
    out->num_active_meetings = b->num_active_meetings;
    out->grids_stack_index = b->grids_stack_index;
    out->schema_stack_index = b->schema_stack_index;
    out->grids_stack_capacity = b->grids_stack_capacity;
    out->schema_stack_capacity = b->schema_stack_capacity;
    out->grid_capacity = b->grid_capacity;
    out->x_buffer = h->config->x_buffer;
    out->y_buffer = h->config->y_buffer;
    out->ms_filter = h->ms_filter;
    out->ms_refine = h->ms_refine;
    out->ms_meet = h->ms_meet;
    out->ms_schema = h->ms_schema;
}

/* meetings identified by the last step: (key, start, end) in emission order */
uint32_t ref_get_meetings(void *hv, uint64_t *keys, uint32_t *starts, uint32_t *ends, uint32_t cap) {
    ref_handle *h = (ref_handle *)hv;
    workbench *b = h->bench;
    uint32_t n = b->kv_count;
    uint32_t lim = h->config->num_objects * 10;
    if (n > lim) n = lim;
    if (n > cap) n = cap;
    for (uint32_t i = 0; i < n; ++i) {
        keys[i] = b->h_meetings_ps[i].key;
        starts[i] = b->h_meetings_ps[i].start;
        ends[i] = b->h_meetings_ps[i].end;
    }
    return b->kv_count;
}

/* raw copies of the schema (QTSchema records), stacks and grid counters */
uint32_t ref_schema_record_size(void) { return (uint32_t)sizeof(QTSchema); }

void ref_get_schema(void *hv, void *schema_out, uint32_t *schema_stack_out, uint32_t *grids_stack_out,
                    uint32_t *grid_counter_out) {
    ref_handle *h = (ref_handle *)hv;
    workbench *b = h->bench;
    if (schema_out) memcpy(schema_out, b->schema, sizeof(QTSchema) * (size_t)b->schema_stack_capacity);
    if (schema_stack_out) memcpy(schema_stack_out, b->schema_stack, sizeof(uint) * (size_t)b->schema_stack_capacity);
    if (grids_stack_out) memcpy(grids_stack_out, b->grids_stack, sizeof(uint) * (size_t)b->grids_stack_capacity);
    if (grid_counter_out) memcpy(grid_counter_out, b->grid_counter, sizeof(uint) * (size_t)b->grids_stack_capacity);
}

/* the reference's bucket table (key, start, end) after the last step */
void ref_get_buckets(void *hv, uint64_t *keys, uint32_t *starts, uint32_t *ends) {
    ref_handle *h = (ref_handle *)hv;
    workbench *b = h->bench;
    for (size_t i = 0; i < h->config->num_meeting_buckets; ++i) {
        keys[i] = b->meeting_buckets[i].key;
        starts[i] = b->meeting_buckets[i].start;
        ends[i] = b->meeting_buckets[i].end;
    }
}

/* the reference's degree_per_meter_longitude (util/util.h:59-66) as compiled here */
double ref_dpm_lon(double lat) { return degree_per_meter_longitude(lat); }

void ref_destroy(void *hv) {
    ref_handle *h = (ref_handle *)hv;
    delete[] h->points;
    /* workbench::clear() (tracing/workbench.cpp:62-73) walks data[0..499] but
     * the constructor only initialises data[0..99], so it frees garbage.  Free
     * the arena buffers claim_space() made through their public pointers. */
    workbench *b = h->bench;
    free(b->grids); free(b->grid_counter); free(b->grids_stack); free(b->schema); free(b->schema_stack);
    free(b->grid_check); free(b->meeting_buckets); free(b->h_keys); free(b->search_single_list);
    free(b->search_multi_pid); free(b->search_multi_list); free(b->h_longer_edges); free(b->ctbs);
    free(b->h_meetings_ps); free(b->active_meeting_count_ps);
    for (uint32_t i = 0; i < h->config->MemTable_capacity; ++i) {
        free(b->h_bitmaps[i]); free(b->h_bitmap_mbrs[i]); free(b->h_sids[i]); free(b->h_CTF_capacity[i]);
        free(b->h_ctfs[i]); free(b->h_oversize_buffers[i].keys); free(b->h_oversize_buffers[i].boxes);
        free(b->h_oversize_buffers[i].o_bitmaps);
    }
    free(b->h_bitmaps); free(b->h_bitmap_mbrs); free(b->h_sids); free(b->h_CTF_capacity);
    free(b->h_oversize_buffers); free(b->h_ctfs);
    delete h->bench;
    delete h->part;
    delete h->config;
    delete h;
}

} /* extern "C" */
