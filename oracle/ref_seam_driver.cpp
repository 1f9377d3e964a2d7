/*
 * ref_seam_driver.cpp -- the reference's GPU-branch step loop around the seam
 * shim, for tests.
 *
 * TEST INFRASTRUCTURE ONLY.  tests/test_shim.py compiles this with the
 * reference's own tracing sources (process.cpp built with -DUSE_GPU, whose
 * straight_dump writes the store files, and the workbench, partitioner and
 * store classes), the shim glint_pipeline_gb300/shim/glint_ref_shim.cpp and
 * a libglint: the real one, or oracle/fake_glint.c where no GPU is present.
 *
 * The sequence follows tracer::process (tracing/process.cpp:401-612) with
 * config->gpu set: the schema is built once from the first step's points by
 * partitioner::build_schema, the workbench gets mbr, end_time_min,
 * start_time_min/max and dProbFalse, cuda_create_device_bench runs once;
 * every step is reset(), points, cur_time, process_with_gpu, then the
 * search_single -> search_multi hand-over of :476-489, and once
 * MemTable_count reaches MemTable_capacity / 2, end_time_max = cur_time and
 * straight_dump (:549-585; with MemTable_capacity 2 the loop returns there).
 */
#include <cstdint>
#include <cstring>
#include <string>

#include <cstdio>
#include <cstdlib>

#include "tracing/generator.h"
#include "tracing/partitioner.h"
#include "tracing/workbench.h"
#include "cuda/mygpu.h"

workbench *cuda_create_device_bench(workbench *bench, gpu_info *gpu);
void process_with_gpu(workbench *bench, workbench *d_bench, gpu_info *gpu);
void *straight_dump(void *arg);

/* process.cpp's tracer also reaches the reference's GPU enumeration and its
 * map-based generator, which this driver never calls (it builds the
 * workbench itself and is handed the points); they are defined here so that
 * the library links without the reference's CUDA sources and Map data. */
static void never(const char *what) {
    std::fprintf(stderr, "ref_seam_driver: %s is not available in this driver\n", what);
    std::abort();
}
vector<gpu_info *> get_gpus() {
    never("get_gpus");
    return {};
}
void gpu_info::print() { never("gpu_info::print"); }
gpu_info::~gpu_info() {}
void trace_generator::generate_trace(Point *) { never("trace_generator::generate_trace"); }
trace_generator::~trace_generator() {}

extern "C" {

struct seam_config {
    uint32_t num_objects, grid_capacity, min_meet_time, max_meet_time, CTF_count, start_time;
    uint64_t num_meeting_buckets;
    uint64_t kv_restriction;
    double reach_distance;
    double dProbFalse;
    char raid_path[24];            /* configuration::raid_path (SSTables go to <raid_path>0 and 1) */
    char meta_path[24];            /* configuration::CTB_meta_path */
};

struct seam {
    configuration *config;
    partitioner *part;
    workbench *bench, *d_bench;
    Point *points;
    int dumped;
};

void *seam_create(const seam_config *sc, const double *mbr4, const double *points_xy) {
    seam *s = new seam();
    configuration *c = new configuration();
    c->num_objects = sc->num_objects;
    c->num_threads = 1;
    c->grid_capacity = sc->grid_capacity;
    c->zone_capacity = sc->grid_capacity;
    c->min_meet_time = sc->min_meet_time;
    c->max_meet_time = sc->max_meet_time;
    c->num_meeting_buckets = sc->num_meeting_buckets;
    c->reach_distance = sc->reach_distance;
    c->start_time = sc->start_time;
    c->gpu = true;
    c->MemTable_capacity = 2;
    c->CTF_count = sc->CTF_count;
    c->update();                   /* split_num = sqrt(CTF_count) and the kv sizes */
    c->kv_restriction = (uint)sc->kv_restriction;
    c->kv_capacity = (uint)(sc->kv_restriction + 1000000);
    c->oversize_buffer_capacity = (uint)(sc->kv_restriction + 1000000);
    c->file_size = 10;             /* indexes area_reistriction[], and names the files */
    std::memcpy(c->raid_path, sc->raid_path, sizeof(c->raid_path));
    std::memcpy(c->CTB_meta_path, sc->meta_path, sizeof(c->CTB_meta_path));
    s->config = c;
    box b(mbr4[0], mbr4[1], mbr4[2], mbr4[3]);
    s->part = new partitioner(b, c);
    s->points = new Point[sc->num_objects];
    std::memcpy((void *)s->points, points_xy, sizeof(Point) * (size_t)sc->num_objects);
    workbench *bench = s->part->build_schema(s->points, sc->num_objects);
    bench->mbr = b;
    bench->end_time_min = c->start_time + c->min_meet_time;
    bench->start_time_min = (1ULL << 32) - 1;
    bench->start_time_max = 0;
    bench->dProbFalse = sc->dProbFalse;
    s->bench = bench;
    s->d_bench = cuda_create_device_bench(bench, nullptr);
    s->dumped = 0;
    return s;
}

/* one step; returns 1 when this step ended with straight_dump */
int seam_step(void *h, const double *points_xy, uint32_t cur_time) {
    seam *s = (seam *)h;
    workbench *bench = s->bench;
    std::memcpy((void *)s->points, points_xy, sizeof(Point) * (size_t)s->config->num_objects);
    bench->reset();
    bench->points = s->points;
    bench->cur_time = cur_time;
    process_with_gpu(bench, s->d_bench, nullptr);
    if (bench->search_multi) bench->search_multi = false;
    if (bench->search_single) {
        bench->search_single = false;
        bench->search_multi = true;
        bench->search_multi_length = bench->single_find_count;
        for (uint32_t i = 0; i < bench->single_find_count; i++)
            bench->search_multi_pid[i] = bench->search_single_list[i].target;
    }
    if (bench->MemTable_count == bench->config->MemTable_capacity / 2) {
        bench->end_time_max = bench->cur_time;
        straight_dump((void *)bench);
        s->dumped = 1;
        return 1;
    }
    return 0;
}

void seam_search_single(void *h, uint32_t pid) {
    seam *s = (seam *)h;
    s->bench->search_single = true;
    s->bench->search_single_pid = pid;
}

/* the last step's search results: which = 0 single, 1 multi; records as
 * (pid, target, start, end, low0, low1, high0, high1) */
uint32_t seam_search_results(void *h, int which, void *out, uint32_t cap) {
    seam *s = (seam *)h;
    workbench *b = s->bench;
    const uint32_t n = which ? b->multi_find_count : b->single_find_count;
    search_info_unit *src = which ? b->search_multi_list : b->search_single_list;
    for (uint32_t i = 0; i < n && i < cap; ++i) {
        search_info_unit u = src[i];
        if (!which) u.pid = b->search_single_pid;
        std::memcpy((char *)out + sizeof(search_info_unit) * i, &u, sizeof(u));
    }
    return n;
}

void seam_counts(void *h, uint64_t *out6) {
    seam *s = (seam *)h;
    workbench *b = s->bench;
    out6[0] = b->grid_check_counter;
    out6[1] = b->num_taken_buckets;
    out6[2] = b->num_active_meetings;
    out6[3] = b->MemTable_count;
    out6[4] = b->ctb_count;
    out6[5] = b->end_time_min;
}

}  // extern "C"
