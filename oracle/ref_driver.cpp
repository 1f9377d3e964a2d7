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

/* ---- the reference's own CTF encoding (tracing/step_merge.cpp), used to pin
 * the flush restatement's bit widths, box quantisation and key layout ---- */

/* CTF::get_ctf_bits for a CTF box; bits = key_bit, id_bit, duration_bit,
 * end_bit, low_x_bit, low_y_bit, edge_bit, mbr_bit, x_grid, y_grid */
void ref_ctf_bits(const float *ctf_mbr4, const double *map4, uint32_t num_objects, uint32_t max_meet_time,
                  uint16_t *bits, uint32_t *bitmap_size) {
    CTF c;
    c.ctf_mbr.low[0] = ctf_mbr4[0];
    c.ctf_mbr.low[1] = ctf_mbr4[1];
    c.ctf_mbr.high[0] = ctf_mbr4[2];
    c.ctf_mbr.high[1] = ctf_mbr4[3];
    box map(map4[0], map4[1], map4[2], map4[3]);
    configuration cfg;
    cfg.num_objects = num_objects;
    cfg.max_meet_time = max_meet_time;
    c.get_ctf_bits(map, &cfg);
    bits[0] = c.key_bit; bits[1] = c.id_bit; bits[2] = c.duration_bit; bits[3] = c.end_bit;
    bits[4] = c.low_x_bit; bits[5] = c.low_y_bit; bits[6] = c.edge_bit; bits[7] = c.mbr_bit;
    bits[8] = c.x_grid; bits[9] = c.y_grid;
    *bitmap_size = c.ctf_bitmap_size;
}

static void ref_ctf_from(CTF &c, const float *ctf_mbr4, const uint16_t *bits) {
    c.ctf_mbr.low[0] = ctf_mbr4[0];
    c.ctf_mbr.low[1] = ctf_mbr4[1];
    c.ctf_mbr.high[0] = ctf_mbr4[2];
    c.ctf_mbr.high[1] = ctf_mbr4[3];
    c.key_bit = bits[0]; c.id_bit = bits[1]; c.duration_bit = bits[2]; c.end_bit = bits[3];
    c.low_x_bit = bits[4]; c.low_y_bit = bits[5]; c.edge_bit = bits[6]; c.mbr_bit = bits[7];
    c.x_grid = bits[8]; c.y_grid = bits[9];
}

/* CTF::serial_mbr of a box inside the CTF box */
uint64_t ref_serial_mbr(const float *ctf_mbr4, const uint16_t *bits, const float *box4) {
    CTF c;
    ref_ctf_from(c, ctf_mbr4, bits);
    f_box b;
    b.low[0] = box4[0];
    b.low[1] = box4[1];
    b.high[0] = box4[2];
    b.high[1] = box4[3];
    return c.serial_mbr(&b);
}

/* CTF::serial_key, as 16 little-endian bytes */
void ref_serial_key(const float *ctf_mbr4, const uint16_t *bits, uint64_t pid, uint64_t target, uint64_t duration,
                    uint64_t end, uint64_t value_mbr, uint8_t *out16) {
    CTF c;
    ref_ctf_from(c, ctf_mbr4, bits);
    __uint128_t k = c.serial_key(pid, target, duration, end, (__uint128_t)value_mbr);
    std::memcpy(out16, &k, 16);
}

/* CTF::binary_search + the key walk of search_SSTable over packed keys:
 * the first index holding oid and the number of consecutive keys of oid */
int ref_ctf_find(const float *ctf_mbr4, const uint16_t *bits, const uint8_t *keys, uint32_t n, uint32_t oid,
                 uint32_t *count) {
    CTF c;
    ref_ctf_from(c, ctf_mbr4, bits);
    c.CTF_kv_capacity = n;
    c.keys = reinterpret_cast<__uint128_t *>(const_cast<uint8_t *>(keys));
    const int find = c.binary_search(oid);
    uint32_t k = 0;
    if (find >= 0) {
        __uint128_t t = 0;
        for (uint32_t i = (uint32_t)find; i < n; ++i) {
            t = 0;
            std::memcpy(&t, keys + (size_t)i * c.key_bit / 8, c.key_bit / 8);
            if (c.ctf_get_key_oid(t) != oid) break;
            ++k;
        }
    }
    *count = k;
    c.keys = nullptr;
    return find;
}

/* ---- the reference's readers of a dumped block (workbench::load_CTB_meta,
 * load_CTF_meta, load_CTF_keys, tracing/workbench.cpp:302-325, 639-695), used
 * to pin the file layout of glint_store_write ---- */
struct ref_store {
    configuration *config;
    workbench *bench;
    uint32_t ctb;
};

/* meta_prefix = <meta_path>/<prefix>; raid_path and keys_prefix go into the
 * reference's fixed-size fields (at most 23 characters) */
void *ref_store_load(const char *meta_prefix, const char *raid_path, const char *keys_prefix, uint32_t ctb,
                     uint32_t num_objects, uint32_t CTF_count) {
    ref_store *h = new ref_store();
    configuration *c = new configuration();
    c->num_objects = num_objects;
    c->CTF_count = CTF_count;
    std::strncpy(c->raid_path, raid_path, sizeof(c->raid_path) - 1);
    workbench *b = new workbench(c);
    b->bit_count = 256 * 256;
    std::strncpy(b->keys_file_prefix, keys_prefix, sizeof(b->keys_file_prefix) - 1);
    b->ctbs = new CTB[ctb + 1];
    b->load_CTB_meta(meta_prefix, (int)ctb);
    for (uint32_t j = 0; j < CTF_count; ++j) b->load_CTF_keys(ctb, j);
    h->config = c;
    h->bench = b;
    h->ctb = ctb;
    return h;
}

/* what the reference read: sids, the oversize buffer (count, times, keys,
 * boxes, bitmap), every CTF's fields in the 64-byte metadata layout of the
 * store, its bitmap bytes (ctf_bitmap_size each, slots of 8192) and keys */
void ref_store_get(void *hv, uint16_t *sids, uint32_t *o_count_times, uint8_t *o_keys, float *o_boxes,
                   uint8_t *o_bitmap, uint8_t *ctf_meta64, uint8_t *bitmaps, uint8_t *keys) {
    ref_store *h = (ref_store *)hv;
    CTB &t = h->bench->ctbs[h->ctb];
    const uint32_t N = h->config->num_objects, C = h->config->CTF_count;
    std::memcpy(sids, t.sids, sizeof(uint16_t) * N);
    const oversize_buffer &o = t.o_buffer;
    o_count_times[0] = o.oversize_kv_count;
    o_count_times[1] = o.start_time_min;
    o_count_times[2] = o.start_time_max;
    o_count_times[3] = o.end_time_min;
    o_count_times[4] = o.end_time_max;
    std::memcpy(o_keys, o.keys, 16 * (size_t)o.oversize_kv_count);
    std::memcpy(o_boxes, o.boxes, sizeof(f_box) * (size_t)o.oversize_kv_count);
    std::memcpy(o_bitmap, o.o_bitmaps, 256 * 256 / 8);
    size_t at = 0;
    for (uint32_t j = 0; j < C; ++j) {
        const CTF &f = t.ctfs[j];
        uint8_t *m = ctf_meta64 + 64 * (size_t)j;
        std::memset(m, 0, 64);
        std::memcpy(m, &f.ctf_mbr, 16);
        const uint32_t u[6] = {f.CTF_kv_capacity, f.start_time_min, f.start_time_max, f.end_time_min, f.end_time_max,
                               f.ctf_bitmap_size};
        std::memcpy(m + 16, u, sizeof(u));
        const uint16_t b[10] = {f.key_bit, f.id_bit, f.duration_bit, f.end_bit, f.low_x_bit,
                                f.low_y_bit, f.edge_bit, f.mbr_bit,  f.x_grid,  f.y_grid};
        std::memcpy(m + 40, b, sizeof(b));
        std::memcpy(bitmaps + (size_t)j * (256 * 256 / 8), f.bitmap, f.ctf_bitmap_size);
        const size_t n = (size_t)f.key_bit / 8 * f.CTF_kv_capacity;
        std::memcpy(keys + at, f.keys, n);
        at += n;
    }
}

/* the reference's lookup of one object in the loaded block, as
 * id_search_in_CTB routes it (tracing/workbench.cpp:397-429): sid 0 -> none,
 * sid 1 -> oversize_buffer::search_buffer, else CTF::binary_search and the
 * walk over the object's keys; returns the number of keys of oid */
uint32_t ref_store_find(void *hv, uint32_t oid) {
    ref_store *h = (ref_store *)hv;
    CTB &t = h->bench->ctbs[h->ctb];
    const uint16_t sid = t.sids[oid];
    if (sid == 0) return 0;
    if (sid == 1) {
        time_query tq;
        atomic<long long> cnt(0);
        return t.o_buffer.search_buffer(oid, &tq, false, cnt, nullptr);
    }
    CTF &f = t.ctfs[sid - 2];
    const int find = f.binary_search(oid);
    if (find < 0) return 0;
    uint32_t k = 0;
    const uint8_t *data = reinterpret_cast<const uint8_t *>(f.keys);
    for (uint32_t i = (uint32_t)find; i < f.CTF_kv_capacity; ++i) {
        __uint128_t v = 0;
        std::memcpy(&v, data + (size_t)i * f.key_bit / 8, f.key_bit / 8);
        if (f.ctf_get_key_oid(v) != oid) break;
        ++k;
    }
    return k;
}

void ref_store_free(void *hv) {
    ref_store *h = (ref_store *)hv;
    if (!h) return;
    /* the loaded arrays belong to the CTB and CTF objects (new[]); the rest
     * of the workbench was never allocated */
    delete[] h->bench->ctbs;
    h->bench->ctbs = nullptr;
    delete h->bench;
    delete h->config;
    delete h;
}

/* ---- the reference's compaction (merge_dump, tools/compaction.cpp:729-1215),
 * built from the tool's own source with its main() renamed ---- */
int ref_compact(const char *meta_prefix, const char *raid_path, const char *keys_prefix, uint32_t count,
                uint32_t num_objects, uint32_t CTF_count, const double *map4, uint32_t max_meet_time,
                uint32_t split_num, const char *out_meta_path);

} /* extern "C" */

void *merge_dump(workbench *bench, uint start_ctb, uint merge_ctb_count, vector<vector<key_info>> &keys_with_sid,
                 vector<vector<f_box>> &mbrs_with_sid, vector<vector<uint>> &invert_index,
                 vector<pair<vector<key_info>, vector<f_box>>> &objects_map, vector<object_info> &str_list);

/* serialize_mbr (cuda/geometry.cu:162-172) lives in the GPU sources, which g++
 * does not build; the compaction tool calls it only with its CTF's own box,
 * for which CTF::serial_mbr (tracing/step_merge.cpp:290-310) is the same
 * arithmetic */
uint64_t serialize_mbr(f_box *b, f_box *bitmap_mbr, CTF *ctf) {
    (void)bitmap_mbr;
    return ctf->serial_mbr(b);
}

/* load_meta (tracing/process.cpp:213-236) is called only by the tool's own
 * main(), which is never run here */
workbench *load_meta(const char *, uint, uint) { return nullptr; }

/* blocks 0 .. count-1 read from <meta_prefix>_CTB<i> and their SSTables, as
 * load_meta does, then merged by merge_dump as the tool's main() calls it;
 * the result goes to <out_meta_path><2 count>G_CTB0 / _STcL0-<i> and
 * <raid_path><i % 2>/<2 count>G_SSTable_0-<i> */
extern "C" int ref_compact(const char *meta_prefix, const char *raid_path, const char *keys_prefix, uint32_t count,
                           uint32_t num_objects, uint32_t CTF_count, const double *map4, uint32_t max_meet_time,
                           uint32_t split_num, const char *out_meta_path) {
    configuration *c = new configuration();
    c->num_objects = num_objects;
    c->CTF_count = CTF_count;
    c->split_num = split_num;
    c->G_bytes = 2 * count;       /* the output prefix is "<G_bytes>G" */
    c->max_meet_time = max_meet_time;
    c->num_threads = 1;
    std::strncpy(c->raid_path, raid_path, sizeof(c->raid_path) - 1);
    std::strncpy(c->CTB_meta_path, out_meta_path, sizeof(c->CTB_meta_path) - 1);
    workbench *b = new workbench(c);
    b->bit_count = 256 * 256;
    /* merge_dump ORs bitmaps_size bytes of each source oversize bitmap, which
     * holds bit_count / 8; only the first bit_count / 8 are written out, so
     * the read is kept inside the buffers */
    b->bitmaps_size = b->bit_count / 8;
    b->mbr = box(map4[0], map4[1], map4[2], map4[3]);
    std::strncpy(b->keys_file_prefix, keys_prefix, sizeof(b->keys_file_prefix) - 1);
    b->ctbs = new CTB[count];
    for (uint32_t i = 0; i < count; ++i) b->load_CTB_meta(meta_prefix, (int)i);
    const uint new_count = split_num * split_num;
    vector<object_info> str_list(num_objects);
    vector<vector<key_info>> keys_with_sid(new_count);
    vector<vector<f_box>> mbrs_with_sid(new_count);
    vector<vector<uint>> invert_index(new_count);
    vector<pair<vector<key_info>, vector<f_box>>> objects_map(num_objects);
    merge_dump(b, 0, count, keys_with_sid, mbrs_with_sid, invert_index, objects_map, str_list);
    delete[] b->ctbs;
    b->ctbs = nullptr;
    delete b;
    delete c;
    return 0;
}
