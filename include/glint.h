/*
 * glint.h -- C ABI of the GB300-native GLINT contact-tracing step.
 *
 * This is the drop-in boundary for the reference's per-timestep GPU seam:
 *
 *   workbench *cuda_create_device_bench(workbench *bench, gpu_info *gpu);
 *       declared tracing/process.cpp:373-374, defined cuda/geometry.cu:1395-1565
 *       -> glint_create()
 *   void process_with_gpu(workbench *bench, workbench *d_bench, gpu_info *gpu);
 *       declared tracing/process.cpp:375, defined cuda/geometry.cu:1573-2218,
 *       called once per timestep at tracing/process.cpp:462
 *       -> glint_step() / glint_step_device()
 *
 * and, on the CPU side, for workbench::filter / reachability /
 * update_meetings / update_schema (tracing/workbench.h:311-313, 339), whose
 * results (the meetings identified each step, tracing/meeting.cpp:11-24) are
 * returned by glint_meetings().  The flush of finished meetings into the
 * sorted key-value + bitmap store (cuda/geometry.cu:1752-2135,
 * tracing/step_merge.cpp:132-186) is glint_flush(); contact-trace queries
 * against that store are glint_query_batch().
 *
 * Plain pointers and sizes only.  Every call returns a status instead of
 * exiting (the reference's CUDA_SAFE_CALL exits, cuda/cuda_util.cuh:19-27).
 * A context owns its CUDA stream and device memory; input buffers are
 * borrowed for the duration of a call.  One context per host thread.
 */
#ifndef GLINT_H_
#define GLINT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLINT_ABI_VERSION 1

typedef enum glint_status {
    GLINT_OK = 0,
    GLINT_ERR_INVALID_ARGUMENT = 1,
    GLINT_ERR_CUDA = 2,
    GLINT_ERR_OUT_OF_MEMORY = 3,
    GLINT_ERR_CAPACITY = 4,      /* a fixed-size device buffer overflowed; see error_flags */
    GLINT_ERR_UNSUPPORTED = 5,
    GLINT_ERR_STATE = 6,
    GLINT_ERR_NO_DEVICE = 7
} glint_status;

/* error_flags bits (glint_step_stats.error_flags) */
#define GLINT_EF_CHECKS_OVERFLOW     0x0001u /* cross-leaf check buffer full */
#define GLINT_EF_NEW_OVERFLOW        0x0002u /* per-step new-contact buffer full */
#define GLINT_EF_TABLE_FULL          0x0004u /* meeting table probe found no empty slot */
#define GLINT_EF_LOG_OVERFLOW        0x0008u /* device meeting log full */
#define GLINT_EF_SCHEMA_STACK        0x0010u /* schema or grid stack exhausted */
#define GLINT_EF_SEGMENT_TOO_LARGE   0x0020u /* a leaf holds more objects than the sorter supports */
#define GLINT_EF_DUPLICATE_NEW       0x0040u /* internal: a new key was inserted twice */
#define GLINT_EF_DFS_OVERFLOW        0x0080u /* lookup depth beyond the supported tree depth */
#define GLINT_EF_SCHEMA_WINDOW       0x0100u /* schema update took the slow path */
#define GLINT_EF_TREE_DEPTH          0x0200u /* descent deeper than the supported tree depth */
#define GLINT_EF_KV_OVERFLOW         0x0400u /* more keys pending than kv_capacity */
#define GLINT_EF_STORE_DOMAIN        0x0800u /* a flush outside the reference's domain (see glint_flush) */

/* The configuration fields this path reads from the reference's
 * `configuration` (util/config.h:15-114), plus this implementation's own. */
typedef struct glint_config {
    uint32_t num_objects;          /* configuration::num_objects */
    uint32_t grid_capacity;        /* configuration::grid_capacity (50) */
    double grid_amplify;           /* configuration::grid_amplify (2): leaf buffer = amplify*capacity */
    uint64_t num_meeting_buckets;  /* configuration::num_meeting_buckets; 0 -> 2*num_objects (config.h:176-178) */
    double reach_distance;         /* configuration::reach_distance, metres (2) */
    uint32_t min_meet_time;        /* configuration::min_meet_time (5) */
    uint32_t max_meet_time;        /* configuration::max_meet_time (4096) */
    uint32_t schema_update_delay;  /* configuration::schema_update_delay (1) */
    uint32_t dynamic_schema;       /* configuration::dynamic_schema (1) */
    uint32_t phased_lookup;        /* configuration::phased_lookup; only 1 is supported */
    uint32_t start_time;           /* configuration::start_time */
    double x_buffer;               /* configuration::x_buffer; 0 -> reach*dpm_lon(mbr.low.y) (filter.cpp:30) */
    double y_buffer;               /* configuration::y_buffer; 0 -> reach*dpm_lat (filter.cpp:31) */
    uint32_t G_bytes;              /* configuration::G_bytes: kv_restriction = G_bytes*2^25 keys (config.h:77-85) */
    uint32_t CTF_count;            /* configuration::CTF_count (100); must be a square */
    double dProbFalse;             /* workbench::dProbFalse: object-box area above which keys go to the oversize buffer */
    /* ---- this implementation ---- */
    uint32_t precision_mode;       /* 0: FP64 test on every candidate; 1: FP32 leaf-relative guard band */
    uint32_t device;               /* CUDA device ordinal */
    uint64_t new_capacity;         /* per-step new-contact buffer (entries); 0 -> automatic */
    uint64_t check_capacity;       /* cross-leaf check buffer (entries); 0 -> automatic */
    uint64_t meeting_log_capacity; /* meetings kept on device until the next flush; 0 -> automatic */
    uint32_t timing;               /* 1: record per-stage CUDA-event times in glint_step_stats.ms */
    uint32_t auto_flush;           /* 1: flush inside the step once more than kv_restriction keys are
                                      pending, as cuda/geometry.cu:1752 */
    uint32_t split_num;            /* configuration::split_num (10): STR slices per axis */
    uint32_t store_keep;           /* flushed blocks (CTBs) kept on the device for glint_query_batch;
                                      0 -> none; the oldest is dropped first */
    uint64_t kv_restriction;       /* 0 -> G_bytes*2^25 keys (util/config.h:80) */
    uint64_t kv_capacity;          /* key buffer; 0 -> kv_restriction + max(1000000, 4*num_objects)
                                      (util/config.h:81 adds 1000000) */
    uint32_t use_graph;            /* 1: capture the step once as a CUDA graph and replay it (device
                                      input buffer only; per-stage timing off) */
    uint32_t store_host_keep;      /* further blocks kept in page-locked host memory, which the GPU reads
                                      over the host link: the oldest device-kept block moves there when
                                      a new one arrives beyond store_keep; 0 -> none */
    uint32_t refine_chunk;         /* cross-leaf checks per refine work item (the refine tile width);
                                      results do not depend on it; 0 -> 64 */
    uint32_t reserved3;
} glint_config;

typedef struct glint_box {
    double low[2];                 /* lon, lat */
    double high[2];
} glint_box;

/* Same field layout as the reference's QTSchema (index/QTree.h:49-62), 80 bytes,
 * so a caller can pass workbench::schema unchanged. */
typedef struct glint_schema_node {
    uint32_t grid_id;
    int16_t level;
    int16_t type;                  /* 0 INVALID, 1 BRANCH, 2 LEAF */
    int16_t overflow_count;
    int16_t underflow_count;
    double mid_x;
    double mid_y;
    double low[2];
    double high[2];
    uint32_t children[4];
} glint_schema_node;

/* an initial schema as partitioner::build_schema leaves it (filter.cpp:81-91) */
typedef struct glint_schema_init {
    const glint_schema_node *nodes;   /* workbench::schema, schema_stack_capacity records */
    uint32_t num_nodes;               /* records in `nodes` */
    uint32_t schema_stack_index;      /* workbench::schema_stack_index */
    uint32_t grids_stack_index;       /* workbench::grids_stack_index */
    uint32_t reserved;
    const uint32_t *schema_stack;     /* NULL -> identity (workbench.cpp:106-112) */
    const uint32_t *grids_stack;      /* NULL -> identity (workbench.cpp:95-100) */
} glint_schema_init;

/* one identified meeting: pid1 < pid2 (the Cantor pair key's ids), the
 * first and last steps of contact, and the f32 box of both objects over it */
typedef struct glint_meeting {
    uint32_t pid1;
    uint32_t pid2;
    uint32_t start;
    uint32_t end;
    float mbr[4];                  /* low lon, low lat, high lon, high lat */
} glint_meeting;

typedef struct glint_step_stats {
    uint32_t cur_time;
    uint32_t checks;               /* inside + cross-leaf checks (grid_check_counter) */
    uint32_t border_objects;       /* objects that ran the neighbour lookup (filter_list_index) */
    uint32_t cross_checks;
    uint64_t candidates;           /* distance tests evaluated */
    uint64_t contacts;             /* distance tests within reach */
    uint64_t new_keys;             /* contacts whose pair had no entry at the start of the step */
    uint64_t num_taken_buckets;    /* occupied slots before expiry (meeting.cpp:136-139) */
    uint32_t num_active_meetings;  /* entries touched this step (meeting.cpp:141-144) */
    uint32_t meetings;             /* meetings identified this step */
    uint32_t splits;
    uint32_t merges;
    uint32_t leaves;               /* grids_stack_index */
    uint32_t nodes;                /* schema_stack_index */
    uint32_t dropped_objects;      /* objects past a full leaf buffer (filter.cpp:102) */
    uint32_t rechecks;             /* decisions re-taken with the correctly rounded sin */
    uint32_t ambiguous;            /* rechecks whose outcome depended on libm's last bit */
    uint32_t band_pairs;           /* precision mode: pairs inside the FP32 guard band */
    uint32_t error_flags;          /* GLINT_EF_* */
    uint32_t launches;             /* kernels the step launched */
    uint64_t meeting_log_size;     /* meetings written to the device log so far */
    float ms[8];                   /* copy, partition, filter, refine, insert, identify, schema (what is
                                      left of the schema update after identify, beside which it runs),
                                      total */
    uint64_t kv_count;             /* keys pending for the next flush (workbench::kv_count) */
    uint32_t flushed;              /* 1: this step ended with an automatic flush */
    float flush_ms;                /* its device time (not included in ms[7]) */
    uint32_t box_band;             /* filter box tests inside the FP32 guard band (re-taken in FP64) */
    uint32_t reserved1;
} glint_step_stats;

typedef struct glint_ctx glint_ctx;

int glint_abi_version(void);
const char *glint_status_string(glint_status s);
/* sizeof of glint_config, glint_box, glint_schema_node, glint_schema_init,
 * glint_meeting and glint_step_stats, in that order (binding self-check) */
void glint_struct_sizes(uint32_t out[6]);
/* fills a config with the reference's defaults for n objects (util/config.h) */
void glint_config_defaults(glint_config *cfg, uint32_t num_objects);

/* cuda_create_device_bench: allocate device state and upload the initial
 * schema.  `init` may be NULL, in which case the schema is built from
 * first_points (N lon/lat pairs, host memory) with the reference's rule
 * (index/QTree.h:157-185). */
glint_status glint_create(const glint_config *cfg, const glint_box *mbr, const double *first_points,
                          const glint_schema_init *init, glint_ctx **out);
glint_status glint_destroy(glint_ctx *ctx);
const char *glint_last_error(const glint_ctx *ctx);

/* process_with_gpu: one timestep.  points = N (lon, lat) FP64 pairs in host
 * memory, copied in on the context's stream; returns after the step
 * completes, with stats (may be NULL). */
glint_status glint_step(glint_ctx *ctx, const double *points, uint32_t cur_time, glint_step_stats *stats);
/* the same with points already in device memory; enqueues the step on the
 * context's stream and returns without waiting.  d_points must be device (or
 * managed) memory, else GLINT_ERR_INVALID_ARGUMENT before anything is
 * enqueued */
glint_status glint_step_device(glint_ctx *ctx, const double *d_points, uint32_t cur_time);
/* waits for enqueued steps; stats of the last one (may be NULL) */
glint_status glint_sync(glint_ctx *ctx, glint_step_stats *stats);

/* meetings identified by the last step, in bucket order (the order of
 * workbench::h_meetings_ps, tracing/meeting.cpp:147-153); *n receives the count */
glint_status glint_meetings(glint_ctx *ctx, glint_meeting *out, uint64_t cap, uint64_t *n);

/* debugging / parity state: schema records (num_nodes), the free part of the
 * two stacks, and per-grid object counts from the last step's filter */
glint_status glint_get_schema(glint_ctx *ctx, glint_schema_node *nodes, uint32_t *schema_stack, uint32_t *grids_stack,
                              uint32_t *grid_counter, uint32_t *schema_stack_index, uint32_t *grids_stack_index);
/* table contents: key (or 1<<62 when empty) and start per bucket */
glint_status glint_get_buckets(glint_ctx *ctx, uint64_t *keys, uint32_t *starts, float *mbrs);
/* sizes the context was created with */
glint_status glint_get_capacities(const glint_ctx *ctx, uint32_t *schema_capacity, uint32_t *grids_capacity,
                                  uint64_t *buckets);
/* the context's cudaStream_t */
void *glint_stream(glint_ctx *ctx);

/* ---- snapshot and resume -------------------------------------------------
 * The reference's workbench::dump_meta / load_meta (tracing/workbench.cpp:
 * 574-596, tracing/process.cpp:213-236) keep the flushed blocks but not the
 * meetings in progress.  glint_snapshot_save writes, between steps, all the
 * state the next steps read: configuration, schema and free stacks, the
 * occupied buckets of the meeting table, the pending keys of the current
 * window, the last step's meetings, the last flushed store, the kept blocks
 * and the counters.  glint_snapshot_load creates a context from such a file
 * (on `device`, or the saved one when negative) that continues bit for bit
 * as the saved context would. */
glint_status glint_snapshot_save(glint_ctx *ctx, const char *path);
glint_status glint_snapshot_load(const char *path, int device, glint_ctx **out);

/* ---- the reference's trace files ------------------------------------------
 * A trace is stored as files <prefix><st>_<num_objects>.tr, st a multiple of
 * 100, each holding 100 steps of num_objects (lon, lat) doubles, step after
 * step, no header (tools/datagen.cpp:18-26, read by tracer::loadData,
 * tracing/process.cpp:128-144).  glint_trace_open starts a host thread that
 * reads steps [first_step, first_step + num_steps) in order into a ring of
 * `ring` (>= 3) page-locked step buffers ahead of the caller.
 * glint_trace_step waits for step t and returns its points; the two steps
 * most recently returned stay valid (the last may still be in an
 * asynchronous copy such as glint_pipe_submit's), older ones are reused.
 * Failures (a missing or short file) are reported by glint_trace_step, with
 * the message in glint_trace_error. */
typedef struct glint_trace glint_trace;
glint_status glint_trace_open(const char *prefix, uint32_t num_objects, uint32_t first_step, uint32_t num_steps,
                              uint32_t ring, glint_trace **out);
glint_status glint_trace_step(glint_trace *trace, uint32_t t, const double **points);
glint_status glint_trace_close(glint_trace *trace);
const char *glint_trace_error(void);
/* num_steps steps of points (step-major, num_objects (lon, lat) pairs each)
 * from first_step on, into the chunk files of that layout */
glint_status glint_trace_write(const char *prefix, uint32_t num_objects, uint32_t first_step, const double *points,
                               uint32_t num_steps);

/* ---- pipelined stepping from host memory ----------------------------------
 * No counterpart in the reference, whose process_with_gpu copies the points
 * in and the results out around each step (cuda/geometry.cu:1625,
 * 2142-2157).  glint_pipe_submit starts copying a step's points (page-locked
 * memory, glint_host_alloc) on a copy stream into the second of two device
 * buffers while the step before computes, then finishes that step (its
 * statistics and, with auto_flush, its flush, so the flush still falls
 * between the two steps) and queues the new one.  At the end of each step a
 * kernel writes its meetings straight into one of two page-locked result
 * buffers of result_capacity records (0: num_objects).  glint_pipe_result
 * returns a step's statistics and meetings (waiting for it if it is still in
 * flight); they stay valid until the submit two steps later, and only the
 * last finished step can be asked for.  GLINT_ERR_CAPACITY when a step had
 * more meetings than result_capacity (the first result_capacity are there;
 * glint_meetings reads them all).  The context's own stepping calls must not
 * be mixed in while a pipe has a step in flight. */
typedef struct glint_pipe glint_pipe;
glint_status glint_pipe_create(glint_ctx *ctx, uint64_t result_capacity, glint_pipe **out);
glint_status glint_pipe_destroy(glint_pipe *pipe);
glint_status glint_pipe_submit(glint_pipe *pipe, const double *points, uint32_t cur_time);
glint_status glint_pipe_result(glint_pipe *pipe, uint32_t cur_time, glint_step_stats *stats,
                               const glint_meeting **meetings, uint64_t *n);

/* Page-locked host memory (cudaMallocHost) for step inputs and results:
 * glint_step's copy of the points and glint_meetings' copy of the meetings
 * run at the full host link rate from and into it, where pageable memory is
 * staged by the driver.  No counterpart in the reference, which reads traces
 * into pageable buffers (tracing/process.cpp:128-144).  *out is NULL on
 * failure. */
glint_status glint_host_alloc(size_t bytes, void **out);
glint_status glint_host_free(void *p);

/* ---- flush into the sorted key-value + bitmap store ------------------------
 * Every identified meeting whose box lies inside the map becomes two keys
 * (cuda/geometry.cu:665-734): [sid:12][pid:26][target:26][duration:32]
 * [end - end_time_min:32], one per direction, with its f32 box.  A flush
 * (cuda/geometry.cu:1752-2135) partitions objects into CTF_count files by an
 * STR split of their mean positions, sorts the keys, and packs each file's
 * keys into key_bit/8 bytes with the box quantised to the file's extent
 * (tracing/step_merge.cpp:132-186); objects whose meetings lasted longer than
 * max_meet_time or whose area exceeds dProbFalse go to the oversize buffer. */

/* CTF (tracing/step_merge.h) without its two pointers, 64 bytes */
typedef struct glint_ctf_meta {
    float ctf_mbr[4];              /* low lon, low lat, high lon, high lat */
    uint32_t CTF_kv_capacity;
    uint32_t start_time_min, start_time_max;
    uint32_t end_time_min, end_time_max;
    uint32_t ctf_bitmap_size;      /* bytes */
    uint16_t key_bit, id_bit, duration_bit, end_bit, low_x_bit, low_y_bit, edge_bit, mbr_bit, x_grid, y_grid;
    uint32_t reserved;
} glint_ctf_meta;

typedef struct glint_store_info {
    uint64_t kv_count;             /* keys in the CTFs (h_CTF_capacity summed) */
    uint64_t key_bytes;            /* bytes of packed CTF keys (h_keys[offset]) */
    uint32_t oversize_kv_count;    /* oversize_buffer::oversize_kv_count */
    uint32_t oversize_start_time_min, oversize_start_time_max;
    uint32_t oversize_end_time_min, oversize_end_time_max;
    uint32_t sid_count;            /* objects with keys in this window */
    uint32_t oversize_oid_count;
    uint32_t end_time_min;         /* base of the keys' end offsets */
    uint32_t cur_time;             /* step time of the flush (end_time_max) */
    uint32_t reserved;
    uint64_t bits_outside;         /* bitmap bits beyond the bitmap array (dropped) */
} glint_store_info;

/* Flush now: the pending keys become the store (kept on the device until the
 * next flush) and a new window starts at the last step's time.  Returns
 * GLINT_ERR_UNSUPPORTED (GLINT_EF_STORE_DOMAIN) where the reference's own
 * flush leaves its domain: a CTF without keys (its get_ctf_bits asserts),
 * or CTF capacities that do not add up to the key count (meetings longer
 * than max_meet_time shift the reference's CTF ranges). */
glint_status glint_flush(glint_ctx *ctx, glint_store_info *info);
/* No counterpart in the reference (its query tools read blocks from disk).
 * Turns a context into a query server for the blocks it keeps: the meeting
 * table, meeting log and pending-key buffers are released (GLINT_ERR_STATE
 * from then on for steps, flushes, meetings, buckets, active searches,
 * snapshots and pipes), and blocks kept in host memory move onto the device,
 * oldest first, while more than `reserve` bytes of device memory stay free
 * (for the servers' slots).  *blocks_on_device receives how many kept blocks
 * are on the device afterwards.  May be called again to retry the move. */
glint_status glint_serve_only(glint_ctx *ctx, uint64_t reserve, uint32_t *blocks_on_device);
/* The last flush's store, into host arrays (any may be NULL): keys
 * (info.key_bytes), sids (num_objects u16, workbench::h_sids), ctf_capacity
 * and ctfs (CTF_count each), bitmaps (CTF_count * 8192 bytes), the oversize
 * buffer's keys (16-byte little-endian), boxes (4 floats each) and bitmap
 * (8192 bytes). */
glint_status glint_store_read(glint_ctx *ctx, uint8_t *keys, uint16_t *sids, uint32_t *ctf_capacity,
                              glint_ctf_meta *ctfs, uint8_t *bitmaps, void *oversize_keys, float *oversize_boxes,
                              uint8_t *oversize_bitmap, glint_store_info *info);

/* ---- the store on disk, in the reference's file layout ----------------------
 * straight_dump (tracing/process.cpp:254-348) writes a flushed block `ctb` as
 *   <raid_path><i % 2>/<prefix>_SSTable_<ctb>-<i>  CTF i's packed keys
 *   <meta_path>/<prefix>_CTB<ctb>                  CTB record, sids, oversize
 *                                                  keys, boxes and bitmap
 *   <meta_path>/<prefix>_STcL<ctb>-<i>             CTF record + its bitmap
 * (workbench::dump_CTB_meta, CTF::dump_meta: tracing/workbench.cpp:597-614,
 * tracing/step_merge.cpp:644-650), and workbench::load_CTB_meta /
 * load_CTF_meta / load_CTF_keys (tracing/workbench.cpp:302-325, 639-695) read
 * it back; the reference's prefix is "6oversize_<file_size>".  The records
 * have the reference's LP64 layouts (CTF 80 bytes, CTB 128); their pointer
 * fields are written as zero.  Directories must exist. */
typedef struct glint_store_view {
    uint32_t num_objects, CTF_count;
    const uint8_t *keys;               /* packed CTF keys, info.key_bytes */
    const uint16_t *sids;              /* num_objects */
    const glint_ctf_meta *ctfs;        /* CTF_count */
    const uint8_t *bitmaps;            /* CTF_count * 8192 bytes */
    const void *oversize_keys;         /* 16-byte little-endian keys */
    const float *oversize_boxes;       /* 4 floats per key */
    const uint8_t *oversize_bitmap;    /* 8192 bytes */
    glint_store_info info;
} glint_store_view;
/* host arrays (as glint_store_read fills them) into files; no device work */
glint_status glint_store_write(const glint_store_view *store, const char *raid_path, const char *meta_path,
                               const char *prefix, uint32_t ctb);
/* the failure message of the last glint_store_write on this thread */
const char *glint_store_file_error(void);
/* the last flush's store into files */
glint_status glint_store_dump(glint_ctx *ctx, const char *raid_path, const char *meta_path, const char *prefix,
                              uint32_t ctb);
/* files of one block, written here or by the reference, into a block kept
 * on the device for glint_query_batch and servers (the oldest kept block is
 * dropped beyond glint_config.store_keep; GLINT_ERR_STATE when it is 0).  The
 * key end offsets are rebased on the CTF records' end_time_min, the window
 * base the flush wrote there. */
glint_status glint_store_load(glint_ctx *ctx, const char *raid_path, const char *meta_path, const char *prefix,
                              uint32_t ctb);
/* the same for a block of ctf_count CTFs (a compacted block: merge_dump
 * leaves the CTB record's CTF count zero, and the reference's loader takes
 * the count from its configuration, tracing/workbench.cpp:677-681) */
glint_status glint_store_load_ctfs(glint_ctx *ctx, const char *raid_path, const char *meta_path, const char *prefix,
                                   uint32_t ctb, uint32_t ctf_count);

/* ---- the blocks kept on the device ------------------------------------------
 * Kept blocks are numbered from 0, the oldest (glint_store_blocks gives
 * their number). */
typedef struct glint_block_info {
    uint32_t CTF_count;
    uint32_t times[4];             /* the CTB record's start_time_min/max, end_time_min/max */
    uint32_t reserved;
    glint_store_info store;        /* key count and bytes, the oversize buffer's count and times,
                                      end_time_min = base of the key end offsets */
} glint_block_info;
glint_status glint_store_block_info(glint_ctx *ctx, uint32_t block, glint_block_info *info);
/* a kept block into host arrays (any may be NULL), sized as glint_store_read's
 * with CTF_count from glint_store_block_info */
glint_status glint_store_block_read(glint_ctx *ctx, uint32_t block, uint8_t *keys, uint16_t *sids,
                                    glint_ctf_meta *ctfs, uint8_t *bitmaps, void *oversize_keys,
                                    float *oversize_boxes, uint8_t *oversize_bitmap);
/* a kept block into files, in the layout of glint_store_write */
glint_status glint_store_block_dump(glint_ctx *ctx, uint32_t block, const char *raid_path, const char *meta_path,
                                    const char *prefix, uint32_t ctb);

/* ---- compaction of kept blocks ------------------------------------------------
 * merge_dump (tools/compaction.cpp:729-1215) merges `count` consecutive
 * blocks into one of split_num^2 CTFs: every CTF key is parsed, objects are
 * re-partitioned by STR over the middle of their boxes across all merged
 * blocks, each object's keys are ordered by target, CTF limits, bit widths,
 * bitmaps and packed keys are rebuilt, and the oversize buffers are merged in
 * key order.  Its quirks are kept: the last object of the STR order keeps
 * sid 2 and no CTF keys, object lists that STR leaves short are filled with
 * object 0 (whose keys then repeat at the front of those CTFs), and the packed
 * end is the absolute end plus the new CTFs' end_time_min.  Where the
 * reference leaves the order of equivalent objects or keys to std::sort,
 * this keeps them in a stable order (object id; source block and position).
 * Keys are parsed as CTF::parse_key does, except that the object id is read
 * with id_bit bits, as the reference's readers read it: the flush writes its
 * whole (sid, oid) field above the target, so with more than 2^19 objects the
 * packed bytes can keep sid bits above the id, which parse_key would take
 * into the id (and merge_dump would index past its object arrays).
 * The new block takes the place of the merged ones among the kept blocks.
 * GLINT_ERR_UNSUPPORTED (GLINT_EF_STORE_DOMAIN) where merge_dump leaves its
 * domain: no CTF key, a partition size that underflows (too few objects for
 * split_num), a CTF whose bits get_ctf_bits rejects, a key whose object id
 * is beyond num_objects, or a source oversize buffer out of key order. */
typedef struct glint_compact_info {
    uint32_t CTF_count;            /* split_num^2 */
    uint32_t blocks;               /* blocks merged */
    uint64_t kv_count;             /* keys in the new CTFs */
    uint64_t key_bytes;
    uint64_t padding;              /* object-list entries filled with object 0 */
    uint32_t oversize_kv_count;
    uint32_t sid_count;            /* objects placed in CTFs */
    uint32_t x_part, y_part;       /* merge_dump's partition sizes */
    float ms;                      /* device time of the merge */
    uint32_t reserved;
} glint_compact_info;
glint_status glint_store_compact(glint_ctx *ctx, uint32_t first, uint32_t count, uint32_t split_num,
                                 glint_compact_info *info);

/* ---- contact-trace queries over the flushed store ---------------------------
 * The reference reads its store per object (id_search_in_CTB,
 * tracing/workbench.cpp:397-444): the object's sid picks its CTF or the
 * oversize buffer, CTF::binary_search / oversize_buffer::search_buffer find
 * its keys (tracing/step_merge.cpp:67-115, 501-568), and the targets found
 * seed the next hop (search_multi_pid, tracing/process.cpp:476-495).  Here a
 * batch of queries runs on the device over the blocks kept by
 * glint_config.store_keep: hop h+1 expands every object first reached at
 * hop h; a key (pid, target, duration, end) counts when its meeting
 * [end - duration, end] overlaps [t_start, t_end) (start < t_end &&
 * t_start < end; both 0: no window, the reference's abandon = true). */
typedef struct glint_query {
    const uint32_t *seeds;         /* host array */
    uint32_t n_seeds;
    uint32_t hops;                 /* 1..8 */
    uint32_t t_start, t_end;
} glint_query;

typedef struct glint_query_result {
    uint32_t *ids;                 /* host array for the reached objects, or NULL */
    uint64_t cap;                  /* its length */
    uint64_t n;                    /* out: objects reached over all hops (seeds excluded) */
    uint64_t hop_end[8];           /* out: ids[hop_end[h-1] .. hop_end[h]) were first reached at hop h,
                                      each hop's ids ascending */
    uint64_t keys_scanned;         /* out: keys read */
} glint_query_result;

glint_status glint_query_batch(glint_ctx *ctx, const glint_query *queries, uint32_t num_queries,
                               glint_query_result *results);

/* Serving form: continuous batching of contact-trace queries.  A server owns
 * query slots (a visited bitmap and two frontier lists each); the number of
 * slots is min(max_slots, what half of the free device memory holds).  Each
 * glint_server_step admits queued queries into free slots, advances every
 * active query by one hop in one launch, and retires the finished ones, so a
 * query that arrives while others are in flight joins at the next step.  A
 * query's result does not depend on what else is in flight.  The server
 * reads the context's kept store blocks; one host thread drives it, between
 * steps of the context. */
typedef struct glint_server glint_server;
glint_status glint_server_create(glint_ctx *ctx, uint32_t max_slots, glint_server **out);
glint_status glint_server_destroy(glint_server *srv);
uint32_t glint_server_slots(const glint_server *srv);
/* queue a query (its seeds are copied); *ticket identifies it */
glint_status glint_server_submit(glint_server *srv, const glint_query *query, uint64_t *ticket);
/* one admission + hop + retirement round; optional counts after it */
glint_status glint_server_step(glint_server *srv, uint32_t *active, uint32_t *queued);
/* *done = 1 when the query has finished; its result is then written into r
 * (ids up to r->cap) and the ticket is released */
glint_status glint_server_poll(glint_server *srv, uint64_t ticket, glint_query_result *r, int *done);
/* number of flushed blocks currently kept for queries */
uint32_t glint_store_blocks(const glint_ctx *ctx);

/* ---- active contact search --------------------------------------------
 * search_info_unit (tracing/workbench.h:85-88): one active meeting of a
 * listed object. */
typedef struct glint_search_info {
    uint32_t pid;                  /* the listed object */
    uint32_t target;               /* the object it is meeting */
    uint32_t start;                /* first step of the meeting */
    uint32_t end;                  /* the last step's time: the meeting is active */
    float mbr[4];                  /* low lon, low lat, high lon, high lat */
} glint_search_info;

/* The reference's active multi-search (search_multi_pid -> search_multi_list,
 * cuda/geometry.cu:605-663, printed at tracing/process.cpp:465-475), run
 * against the meeting table after the last step: every meeting active at
 * that step that has lasted cur_time - start >= min_meet_time + 1 yields
 * one record per side whose id is listed.  Records come in bucket order, the
 * lower id's side first; a repeated id counts once (the reference appends
 * with an atomic counter, so its order is arbitrary).  pids and out are host
 * arrays; *n receives the number found and the first min(n, cap) records are
 * written.  Waits for the context's stream.  Returns GLINT_ERR_STATE before
 * the first step. */
glint_status glint_active_search(glint_ctx *ctx, const uint32_t *pids, uint32_t npids, glint_search_info *out,
                                 uint64_t cap, uint64_t *n);

/* No counterpart in the reference: glint_active_search for callers that must
 * not allocate device memory on the call (a serving loop, a captured
 * stream).  d_pids (npids ids), d_out (cap records) and d_n (one uint64_t
 * receiving the count) are device arrays; the same records as
 * glint_active_search are written to d_out.  Enqueued on the context's stream
 * (glint_stream); returns without waiting.
 * Scratch: one fixed array of the library per device (2 MB id bitmap +
 * 1 MB of tile counters), whose address is looked up inside every
 * glint_create with that device current (so a context created after a
 * device reset uses the new address); the call itself performs no
 * allocation.  The bitmap is cleared by each call; nothing else needs to
 * start at zero.  Limits: contexts of at most 2^24 objects and 2^30 buckets
 * (GLINT_ERR_UNSUPPORTED otherwise).  Calls that overlap in time on the same
 * device (from any context or stream) share the scratch and race: order them
 * on one stream or synchronise between them. */
glint_status glint_active_search_noalloc(glint_ctx *ctx, const uint32_t *d_pids, uint32_t npids,
                                         glint_search_info *d_out, uint64_t cap, uint64_t *d_n);

/* ---- precision form: the FP32 screen against the FP64 test ---------------
 * No counterpart in the reference, whose distance test is FP64 only
 * (tracing/refinement.cpp:19-31, geometry/geometry.h:40-48).  With
 * precision_mode 1 the refine stage decides each pair with an FP32 screen and
 * re-tests in FP64 only the pairs inside the guard band; this probe measures
 * that screen on the last step's positions.  It samples the pairs (i, i + o),
 * o = 1..32, of leaf-major ranks i = 0, stride, 2 stride, ..., and compares the
 * screen's FP32 distance d32 with the reference's FP64 Point::distance d64
 * and the screen's decision with the FP64 decision.  Works in either
 * precision mode; waits for the context's stream; leaves the step's
 * statistics untouched.  GLINT_ERR_STATE before the first step. */
typedef struct glint_precision_report {
    uint64_t pairs;                /* sampled pairs */
    uint64_t in_band;              /* pairs the screen leaves to the FP64 test */
    uint64_t mismatches;           /* pairs the screen decides against the FP64 test (0 by construction) */
    uint64_t contacts;             /* pairs within reach by the FP64 test */
    double max_abs_err_m;          /* max |d32 - d64| over the sampled pairs, metres */
    double max_abs_err_near_m;     /* the same over pairs with d64 <= 2 r */
    double max_band_m;             /* widest guard band met, as a distance either side of r, metres */
    uint32_t stride;
    uint32_t reserved;
} glint_precision_report;
glint_status glint_precision_probe(glint_ctx *ctx, uint32_t stride, glint_precision_report *out);

/* ---- batching form: many independent regions on one GPU ------------------
 * Each region is a context created from cfgs[r] (per-stage timing off; all on
 * the same device) with its own stream.  glint_batch_step enqueues one
 * timestep of every region for cur_time, reading d_points[r] (device memory,
 * else GLINT_ERR_INVALID_ARGUMENT before anything is enqueued),
 * as one CUDA graph captured at the first step: every region's stages up to
 * the refine stage, one refine launch over the work items of all regions in
 * precision_mode 1 (regions in mode 0 refine on their own streams), then
 * every region's remaining stages.  Keep the same buffers so the graph is
 * reused; it is captured again when a pointer changes.  The call returns
 * without waiting (after the previous timestep is done); glint_batch_sync
 * waits for it and runs each region's automatic flush, filling stats[r] when
 * stats is not NULL.  glint_batch_region gives a region's context for its
 * meetings, store and queries; work queued on a region's stream runs before
 * the batch's next timestep. */
typedef struct glint_batch glint_batch;
glint_status glint_batch_create(uint32_t num_regions, const glint_config *cfgs, const glint_box *mbrs,
                                const double *const *first_points, glint_batch **out);
glint_status glint_batch_destroy(glint_batch *batch);
uint32_t glint_batch_regions(const glint_batch *batch);
glint_ctx *glint_batch_region(glint_batch *batch, uint32_t region);
glint_status glint_batch_step(glint_batch *batch, const double *const *d_points, uint32_t cur_time);
glint_status glint_batch_sync(glint_batch *batch, glint_step_stats *stats);

/* ---- synthetic trajectories on the device (benchmark input) ----
 * params/objects: the generator's parameter block and object states as
 * produced by the host generator (glint_pipeline_gb300/csrc/tracegen.h) */
typedef struct glint_gen glint_gen;
glint_status glint_gen_create(const void *params, uint32_t params_size, const void *objects, uint32_t num_objects,
                              uint32_t object_size, uint32_t first_step, glint_gen **out);
/* advance to the next step and write N (lon, lat) pairs to d_out on `stream` */
glint_status glint_gen_step(glint_gen *g, double *d_out, void *stream);
glint_status glint_gen_destroy(glint_gen *g);

#ifdef __cplusplus
}
#endif

#endif /* GLINT_H_ */
