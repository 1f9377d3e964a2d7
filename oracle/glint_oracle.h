/*
 * glint_oracle.h -- CPU restatement of GLINT's per-timestep contact-tracing
 * path, used ONLY as the test oracle (tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg).  The product never links or calls it.
 *
 * It restates, single-threaded, the reference's CPU stages:
 *   schema build        tracing/filter.cpp:27-93, index/QTree.h:98-311
 *   filter              tracing/filter.cpp:95-111, 130-152, 209-313
 *   reachability        tracing/refinement.cpp:10-85
 *   update_meetings     tracing/meeting.cpp:32-189
 *   update_schema       tracing/filter.cpp:316-449
 * and the GPU path's per-meeting f32 MBR rule (cuda/geometry.cu:82-96,
 * 469-491), which the CPU path lacks but the key-value store needs.
 *
 * Parity pin: tests compare this restatement against the reference's own
 * sources built into oracle/_ref (build_ref.sh) on seeded inputs, and against
 * fixtures in tests/golden generated from that build.
 */
#ifndef GLINT_ORACLE_H_
#define GLINT_ORACLE_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct go_config {
    uint32_t num_objects;
    uint32_t grid_capacity;       /* configuration::grid_capacity (50) */
    uint32_t schema_update_delay; /* configuration::schema_update_delay (1) */
    uint32_t min_meet_time;       /* configuration::min_meet_time (5) */
    uint32_t dynamic_schema;      /* configuration::dynamic_schema (1) */
    uint32_t pad0;
    uint64_t num_meeting_buckets; /* configuration::num_meeting_buckets (2N) */
    double grid_amplify;          /* configuration::grid_amplify (2) */
    double reach_distance;        /* configuration::reach_distance (2 m) */
} go_config;

/* same field layout as the reference's QTSchema (index/QTree.h:49-62), 80 bytes */
typedef struct go_schema {
    uint32_t grid_id;
    int16_t level;
    int16_t type;
    int16_t overflow_count;
    int16_t underflow_count;
    double mid_x;
    double mid_y;
    double low[2];
    double high[2];
    uint32_t children[4];
} go_schema;

enum { GO_INVALID = 0, GO_BRANCH = 1, GO_LEAF = 2 };

typedef struct go_meeting {
    uint64_t key;                 /* Cantor pair of (min id, max id) */
    uint32_t start;
    uint32_t end;
    float mbr[4];                 /* low x, low y, high x, high y (GPU rule) */
} go_meeting;

typedef struct go_counts {
    uint32_t grid_check_counter;
    uint32_t kv_count;            /* meetings identified by the last step */
    uint64_t num_taken_buckets;
    uint32_t num_active_meetings;
    uint32_t grids_stack_index;
    uint32_t schema_stack_index;
    uint32_t grids_stack_capacity;
    uint32_t schema_stack_capacity;
    uint32_t grid_capacity;       /* leaf buffer size = grid_amplify*grid_capacity */
    uint64_t contacts;            /* distance tests that passed in the last step */
    uint64_t candidates;          /* distance tests evaluated in the last step */
    uint32_t n_splits;            /* schema splits in the last step */
    uint32_t n_merges;            /* schema merges in the last step */
    double x_buffer;
    double y_buffer;
    uint32_t range_reruns;        /* slot ranges run again for probes crossing range ends (threads > 1) */
    uint32_t pad1;
} go_counts;

typedef struct go_ctx go_ctx;

/* the reference's geographic helpers (util/util.h:57-70) */
double go_dpm_lon(double latitude);
double go_dpm_lat(void);
uint64_t go_cantor(uint32_t a, uint32_t b);
void go_cantor_inverse(uint64_t z, uint32_t *a, uint32_t *b);

/* builds the initial schema from the first step's points, as
 * partitioner::build_schema does; mbr4 = low x, low y, high x, high y */
go_ctx *go_create(const go_config *cfg, const double *mbr4, const double *points_xy);
/* the same with `threads` host threads for the order-free parts of every
 * step (go_set_threads); results are identical for every thread count */
go_ctx *go_create_threads(const go_config *cfg, const double *mbr4, const double *points_xy, uint32_t threads);
void go_set_threads(go_ctx *c, uint32_t threads);
void go_destroy(go_ctx *c);

/* one timestep: filter, reachability, update_meetings, update_schema */
int go_step(go_ctx *c, const double *points_xy, uint32_t cur_time);

void go_get_counts(const go_ctx *c, go_counts *out);
/* meetings identified by the last step in bucket order; returns the count */
uint32_t go_get_meetings(const go_ctx *c, go_meeting *out, uint32_t cap);
/* raw state for step-by-step comparisons */
void go_get_schema(const go_ctx *c, go_schema *schema, uint32_t *schema_stack, uint32_t *grids_stack,
                   uint32_t *grid_counter);
void go_get_buckets(const go_ctx *c, uint64_t *keys, uint32_t *starts, uint32_t *ends, float *mbrs);

/* search_info_unit (tracing/workbench.h:85-88) */
typedef struct go_search_info {
    uint32_t pid, target, start, end;
    float mbr[4];
} go_search_info;

/* the GPU path's active multi-search (cuda/geometry.cu:605-663) over the
 * bucket table after the last step; records in bucket order; returns the
 * number found (only the first cap are written) */
uint64_t go_active_search(const go_ctx *c, const uint32_t *pids, uint32_t npids, go_search_info *out,
                          uint64_t cap);

/* ---- key generation and flush into the key-value + bitmap store
 * (glint_flush_oracle.c; cuda/geometry.cu:665-734, 739-1107, 1752-2135,
 * tracing/step_merge.cpp:132-186) ---- */
typedef struct go_store_config {
    uint32_t num_objects;
    uint32_t max_meet_time;       /* configuration::max_meet_time (4096) */
    uint32_t CTF_count;           /* configuration::CTF_count (100) */
    uint32_t split_num;           /* configuration::split_num (10) */
    uint32_t first_end_time_min;  /* start_time + min_meet_time (tracing/process.cpp:404) */
    uint32_t pad0;
    double dProbFalse;            /* per-object area cut (tracing/process.cpp:408-411) */
    double mbr[4];                /* map box: low x, low y, high x, high y */
    uint64_t kv_capacity;         /* key buffer size */
} go_store_config;

/* one reported meeting, pid1 < pid2 */
typedef struct go_meeting_rec {
    uint32_t pid1, pid2, start, end;
    float mbr[4];
} go_meeting_rec;

/* CTF (tracing/step_merge.h) without its pointers, 64 bytes */
typedef struct go_ctf_meta {
    float ctf_mbr[4];
    uint32_t CTF_kv_capacity;
    uint32_t start_time_min, start_time_max, end_time_min, end_time_max;
    uint32_t ctf_bitmap_size;
    uint16_t key_bit, id_bit, duration_bit, end_bit, low_x_bit, low_y_bit, edge_bit, mbr_bit, x_grid, y_grid;
    uint32_t reserved;
} go_ctf_meta;

typedef struct go_store_info {
    uint64_t kv_count;            /* keys in the CTFs */
    uint64_t key_bytes;           /* bytes of packed CTF keys */
    uint32_t oversize_kv_count;
    uint32_t oversize_start_time_min, oversize_start_time_max;
    uint32_t oversize_end_time_min, oversize_end_time_max;
    uint32_t sid_count;
    uint32_t oversize_oid_count;
    uint32_t end_time_min;        /* the window's base for key end offsets */
    uint32_t cur_time;
    uint32_t reserved;
    uint64_t bits_outside;        /* bitmap bits past the end of the bitmap array (dropped) */
} go_store_info;

typedef struct go_store go_store;
go_store *go_store_create(const go_store_config *cfg);
void go_store_destroy(go_store *s);
void go_store_add_meetings(go_store *s, const go_meeting_rec *m, uint64_t n);
uint64_t go_store_kv_count(const go_store *s);
/* 0 on success; <0 outside the reference's domain (an empty CTF, key overflow) */
int go_store_flush(go_store *s, uint32_t cur_time, go_store_info *out);
/* the last flush's outputs; o_keys are 16-byte little-endian keys */
void go_store_result(const go_store *s, uint8_t *keys, uint16_t *sids, uint32_t *ctf_capacity, go_ctf_meta *ctfs,
                     uint8_t *bitmaps, void *o_keys, float *o_boxes, uint8_t *o_bitmap);

/* the last flush's sorted 16-byte keys (CTF part, then oversize part) and
 * boxes; returns their number */
uint64_t go_store_sorted(const go_store *s, void *keys, float *boxes);

/* ---- contact-trace queries over the store (glint_query_oracle.c) ---- */
/* one key of the store as a meeting edge */
typedef struct go_edge {
    uint32_t pid, target, start, end;
} go_edge;

/* objects first reached at each of `hops` hops from the seeds over edges
 * overlapping [t_start, t_end) (t_start == t_end == 0: no window), each hop's
 * ids ascending, seeds excluded; hop_end[h] = ids after hop h; returns the
 * total (only the first cap are written) */
uint64_t go_query_bfs(const go_edge *edges, uint64_t n_edges, uint32_t num_objects, const uint32_t *seeds,
                      uint32_t n_seeds, uint32_t t_start, uint32_t t_end, uint32_t hops, uint32_t *out,
                      uint64_t cap, uint64_t *hop_end);

/* correctly rounded sin on [0, pi/2] by a double-double Taylor series; used to
 * check how often libm's sin differs from the correctly rounded value */
double go_sin_cr(double x);

/* CTF::get_ctf_bits on c->ctf_mbr (fills the bit widths, grids and bitmap
 * size); 0 where the reference's asserts fire.  serialize_mbr of a box. */
int go_ctf_bits(go_ctf_meta *c, const double *map4, uint32_t num_objects, uint32_t max_meet_time);
uint64_t go_serialize_box(const float *box4, const go_ctf_meta *c);

/* ---- compaction of stored blocks (glint_compact_oracle.c;
 * tools/compaction.cpp:729-1215) ---- */
/* one source block as the store holds it */
typedef struct go_block {
    uint32_t CTF_count, o_count;
    const uint16_t *sids;          /* num_objects */
    const go_ctf_meta *ctfs;       /* CTF_count */
    const uint8_t *keys;           /* the CTFs' packed keys, one CTF after another */
    const uint8_t *o_keys;         /* o_count 16-byte little-endian keys */
    const float *o_boxes;          /* o_count x 4 */
    const uint8_t *o_bitmap;       /* 8192 bytes */
    uint32_t o_times[4];           /* oversize buffer start_time_min/max, end_time_min/max */
    uint32_t times[4];             /* the CTB record's start_time_min/max, end_time_min/max */
} go_block;

typedef struct go_compaction go_compaction;
/* merges `count` blocks into one of split_num^2 CTFs; 0 on success, < 0
 * where merge_dump leaves its domain (GO_CMP_* below).  std_ties: order
 * equivalent elements as the C++ library's std::sort does (the reference's
 * exact output); 0: keep them in a stable order (the device path's). */
int go_compact(const go_block *blocks, uint32_t count, uint32_t num_objects, const double *map4,
               uint32_t max_meet_time, uint32_t split_num, int std_ties, go_compaction **out);
#define GO_CMP_NO_KEYS (-1)        /* no object has a CTF key */
#define GO_CMP_PARTITION (-2)      /* too few objects for split_num: a partition size underflows */
#define GO_CMP_OID (-3)            /* a decoded object id beyond num_objects */
#define GO_CMP_CTF_BITS (-4)       /* get_ctf_bits asserts (an empty CTF, too many key bits) */
/* sizes[8]: CTF_count, kv_count, key_bytes, o_count, padding (entries of oid
 * 0 that fill the per-CTF object lists), x_part, y_part, sid_count (objects
 * placed in CTFs) */
void go_compact_sizes(const go_compaction *h, uint64_t *sizes);
/* times8: the CTB record's start/end times, then the oversize buffer's */
void go_compact_result(const go_compaction *h, uint8_t *keys, uint16_t *sids, go_ctf_meta *ctfs, uint8_t *bitmaps,
                       void *o_keys, float *o_boxes, uint8_t *o_bitmap, uint32_t *times8);
void go_compact_free(go_compaction *h);

#ifdef __cplusplus
}
#endif
#endif
