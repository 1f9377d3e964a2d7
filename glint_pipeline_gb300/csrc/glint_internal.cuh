/*
 * glint_internal.cuh -- the device-resident state of one context and the
 * host launchers of each per-step stage.
 *
 * HBM layout (N objects, G grid slots, S schema slots, B buckets):
 *   points      double2[N]   lon/lat as given, AoS 16 B per object
 *   obj_*       u32[N]       leaf grid id, last_valid node, leaf node per object
 *   sorted      u32[N]       object ids sorted by (grid id, object id): leaf member lists
 *   sxy         double2[N]   coordinates gathered in that order (leaf tiles)
 *   sipos, sc   [N]          fixed-point coordinates (i64 pair) and screening scale, same order
 *   sfpos, fpos float2[N]    FP32 coordinates (meeting boxes), sorted and by object id
 *   sL          double[N]    degree_per_meter_longitude with CUDA sin (plain form only)
 *   nodes       DNode[S]     64-byte schema records (comparison keys), low corners in
 *                            low[S], fixed-point boxes in ibox[S]
 *   stacks      u32[S], u32[G]  free schema / grid slots (workbench.h:118-128)
 *   qlist/tlist              cross-leaf checks, by querier and by target leaf
 *   tab, stamp  TRec[B], u8[B]  the meeting table (32 B per bucket) and touch stamps
 *   newlist     (key, prio)  contacts whose pair was absent at the start of the step
 *   log         glint_meeting ring of identified meetings
 */
#ifndef GLINT_INTERNAL_CUH_
#define GLINT_INTERNAL_CUH_

#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "glint_device.cuh"

namespace glint {

/* counters shared by the kernels of one step; copied to pinned host memory
 * at the end of each step */
struct DevCounters {
    unsigned int cross_checks;
    unsigned int border_objects;
    unsigned long long candidates;
    unsigned long long contacts;
    unsigned long long new_keys;          /* entries appended to the new list */
    unsigned long long taken;
    unsigned int active;
    unsigned int meetings;
    unsigned int splits;
    unsigned int merges;
    unsigned int dropped;
    unsigned int rechecks;
    unsigned int ambiguous;
    unsigned int band_pairs;
    unsigned int box_band;
    unsigned int error_flags;
    unsigned int n_leaf_work;              /* leaves with at least one object */
    unsigned int work_next;                /* dynamic scheduling cursor */
    unsigned int n_events;                 /* schema events this step */
    unsigned int n_cand;                   /* merge candidates this step */
    unsigned int total_checks;
    unsigned int n_big;                    /* leaf segments sorted by a whole block */
    unsigned int n_extra;                  /* refine work items beyond each leaf's first */
    unsigned int extra_next;               /* their scheduling cursor */
    /* persistent (not cleared per step) */
    unsigned int ssi;                      /* schema_stack_index */
    unsigned int gsi;                      /* grids_stack_index */
    unsigned long long log_head;           /* meetings written to the log so far */
    unsigned long long log_step_begin;     /* log position of this step's first meeting */
    unsigned long long kv_count;           /* keys pending for the next flush */
    unsigned int sid_count;                /* objects with at least one pending key */
    unsigned int oversize_oid_count;
    unsigned int keys_outside;             /* meetings outside the map box (not keyed) */
    unsigned int pad2[3];
    /* this step's parameters, copied in at the start of the step so that a
     * captured step graph reads them from here */
    unsigned int step_time;                /* cur_time */
    unsigned int step_tag;                 /* touch tag of this step (1 or 2) */
    unsigned int end_time_min;             /* base of key end offsets */
    unsigned int pad3;
};
struct StepParams {
    unsigned int step_time, step_tag, end_time_min, pad3;
};
/* bytes cleared at the start of every step */
constexpr size_t kStepCounterBytes = offsetof(DevCounters, ssi);

/* cross-leaf checks per refine work item (refine_common.cuh) */
constexpr uint32_t kCrossChunk = 64;       /* default cross-leaf checks per refine work item */
constexpr size_t kMaxBlockSmem = 232448;   /* dynamic shared memory one block may use on sm_103a (227 KB) */

struct NewEntry {
    unsigned long long key;
    unsigned long long prio;
};

struct SchemaEvent {
    uint32_t node;
    uint32_t kind;        /* 0 split, 1 merge */
};

/* one contact-tracing block (CTB) kept on the device: flushed, loaded from
 * files or compacted */
struct StoreBlock {
    uint8_t *keys = nullptr;               /* packed CTF keys */
    uint64_t key_bytes = 0;
    glint_ctf_meta *ctfs = nullptr;        /* [C] */
    unsigned long long *key_index = nullptr, *byte_index = nullptr; /* [C] */
    uint16_t *sids = nullptr;              /* [N] 0 none, 1 oversize, 2.. CTF + 2 */
    uint32_t *first = nullptr, *count = nullptr; /* [N] each object's keys (in its CTF or the oversize buffer) */
    ulonglong2 *okeys = nullptr;           /* oversize keys, 128-bit */
    float4 *oboxes = nullptr;              /* [o_count] oversize boxes */
    uint8_t *bitmaps = nullptr;            /* [C][8192] CTF bitmaps */
    uint8_t *obitmap = nullptr;            /* [8192] oversize bitmap */
    uint64_t kv = 0, o_count = 0;
    uint32_t end_time_min = 0, end_time_max = 0; /* base of the key end offsets; last step */
    uint32_t C = 0;                        /* CTFs */
    uint32_t o_times[4] = {0, 0, 0, 0};    /* oversize buffer start_time_min/max, end_time_min/max */
    uint32_t rec_times[4] = {0, 0, 0, 0};  /* the CTB record's own start/end time fields */
    uint32_t sid_count = 0, oversize_oid_count = 0;
    bool on_host = false;                  /* arrays in page-locked host memory (read over the host link) */
    uint32_t start_min = 0;                /* no key's meeting starts before this, and none ends after
                                              end_time_max: a query window outside both finds nothing */
    bool spans_known = false;              /* start_min and end_time_max were taken from the keys here
                                              (flushed or merged blocks; not blocks read from files) */
};
void store_block_release(StoreBlock &b);
/* the kept blocks after one was added: the oldest device blocks beyond
 * store_keep move to host memory while fewer than store_host_keep are
 * there; beyond that the oldest block is dropped */
cudaError_t store_blocks_trim(glint_ctx *c);

/* device-side descriptor of a StoreBlock */
struct StoreBlockDev {
    const uint8_t *keys;
    unsigned long long key_bytes;
    const glint_ctf_meta *ctfs;
    const unsigned long long *key_index, *byte_index;
    const uint16_t *sids;
    const uint32_t *first, *count;
    const ulonglong2 *okeys;
    uint32_t end_time_min;
    uint32_t C;
};

struct StepTimers {
    cudaEvent_t ev[9];
    bool created = false;
};

glint_status enqueue_device_step_plain(glint_ctx *c, const double *d_points, uint32_t cur_time);
/* true (and last_error set) when the context was turned to serving only */
bool serve_only_refused(glint_ctx *c, const char *what);

} // namespace glint

struct glint_ctx {
    glint_config cfg;
    glint_box mbr;
    int device = 0;
    cudaStream_t stream = nullptr;
    /* the schema update runs here, beside identify, between two events of
     * the step stream */
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    std::string last_error;

    uint32_t N = 0, G = 0, S = 0, cap = 0;
    uint32_t chunk = 64;        /* cross-leaf checks per refine work item */
    uint64_t B = 0, Bm = 0;
    uint64_t check_cap = 0, new_cap = 0, log_cap = 0;
    uint32_t max_leaf_count = 0;           /* sorter limit for one leaf segment */
    double x_buffer = 0, y_buffer = 0, dpm_lat = 0, band = 0;
    uint64_t step_index = 0;
    uint32_t last_time = 0;

    /* objects */
    double2 *d_pts = nullptr;
    uint32_t *d_obj_gid = nullptr, *d_obj_lv = nullptr, *d_obj_leaf = nullptr;
    uint32_t *d_order = nullptr;           /* processing order of the descent */
    uint32_t *d_grid_count = nullptr;      /* [G+1] */
    uint32_t *d_grid_start = nullptr;      /* [G+1] */
    uint32_t *d_grid_cursor = nullptr;     /* [G] */
    uint32_t *d_sorted = nullptr;          /* [N] */
    uint32_t *d_rank_of = nullptr;         /* [N] sorted position of each object */
    double2 *d_sxy = nullptr;
    double *d_sL = nullptr;                /* [N] sorted L (plain form only) */
    longlong2 *d_sipos = nullptr;          /* [N] sorted fixed-point coordinates */
    float2 *d_sfpos = nullptr;             /* [N] sorted f32 coordinates (meeting boxes) */
    float *d_sc = nullptr;                 /* [N] sorted metres per unit along x */
    float2 *d_fpos = nullptr;              /* [N] f32 coordinates by object id */
    glint::IBox *d_ibox = nullptr;           /* [S] fixed-point node boxes */
    glint::Frame frame;
    uint32_t *d_leaf_work = nullptr;       /* [G] grid ids with objects */

    /* schema */
    glint::DNode *d_nodes = nullptr;
    double2 *d_low = nullptr;
    uint32_t *d_sstack = nullptr;
    uint32_t *d_gstack = nullptr;
    uint8_t *d_split = nullptr;            /* [S] per-slot event flags */
    uint32_t *d_evscan = nullptr;          /* [S] candidate leaf-children sums */
    uint32_t *d_cand = nullptr;            /* [S] merge candidates */
    uint32_t *d_newgid = nullptr;          /* [S] grid id a merged node takes */
    uint32_t *d_events = nullptr;          /* [S+1] per-slot event indicator */
    uint32_t *d_evpos = nullptr;           /* [S+1] its exclusive scan */
    uint32_t *d_evlist = nullptr;          /* [S] event slots in slot order */
    uint4 *d_evdata = nullptr;             /* [2S] per-event replay data */
    int32_t *d_evlevel = nullptr;          /* [S] stack level before each event */
    uint32_t *d_big = nullptr;             /* [G] leaves sorted by a whole block */

    /* filter */
    uint32_t *d_qcount = nullptr, *d_qstart = nullptr, *d_qlist = nullptr;
    uint32_t *d_qtmp = nullptr;            /* [N*8] first targets of each border object */
    uint32_t *d_tcount = nullptr, *d_tstart = nullptr, *d_tcursor = nullptr;
    uint2 *d_tlist = nullptr;

    /* table */
    glint::TRec *d_tab = nullptr;
    uint8_t *d_stamp = nullptr;
    uint32_t *d_newline = nullptr;   /* one bit per 4 slots filled this step */
    glint::NewEntry *d_new = nullptr;
    uint2 *d_rextra = nullptr;             /* refine work items (leaf, chunk of cross checks) */
    uint64_t rextra_cap = 0;
    uint32_t *d_tile_cnt = nullptr, *d_tile_off = nullptr;
    uint64_t n_tiles = 0;

    /* output */
    glint_meeting *d_log = nullptr;

    /* key-value store (k_flush.cu) */
    uint64_t kv_cap = 0, kv_restriction = 0;
    uint32_t end_time_min = 0;
    ulonglong2 *d_keys = nullptr, *d_keys2 = nullptr;   /* 128-bit keys, pending / sorted */
    float4 *d_kvbox = nullptr, *d_kvbox2 = nullptr;
    uint32_t *d_same = nullptr;            /* [N] same_pid_count */
    uint4 *d_obox = nullptr;               /* [N] o_boxs */
    uint16_t *d_sids = nullptr, *d_sids_out = nullptr;
    uint8_t *d_over = nullptr;
    uint32_t *d_oids = nullptr, *d_oids2 = nullptr;
    unsigned long long *d_mid = nullptr, *d_mid2 = nullptr;
    uint32_t *d_gcount = nullptr, *d_gstart = nullptr, *d_segof = nullptr, *d_segcur = nullptr, *d_segbig = nullptr;
    uint32_t *d_ctf_cap = nullptr, *d_ctf_n = nullptr;
    glint_ctf_meta *d_ctfs = nullptr;
    unsigned long long *d_ctf_lo = nullptr, *d_ctf_byte = nullptr;
    uint8_t *d_ctf_keys = nullptr, *d_bitmaps = nullptr, *d_obitmap = nullptr;
    unsigned long long *d_fmisc = nullptr;
    void *d_rs_tmp = nullptr;
    uint2 *d_place = nullptr;              /* [N] the key scatter's per-object placement records */
    glint_store_info store;
    std::vector<uint32_t> store_ctf_cap;
    bool store_valid = false;
    bool serve_only = false;    /* glint_serve_only: the step state is gone, the kept blocks remain */
    ulonglong2 *store_keys_ptr = nullptr;
    float4 *store_boxes_ptr = nullptr;
    uint64_t store_kv = 0;
    uint32_t flushes = 0;
    std::vector<glint::StoreBlock> ctbs;   /* flushed blocks kept for queries, oldest first */
    cudaMemPool_t compact_pool = nullptr;  /* compaction scratch; stays mapped between merges */
    glint_server *server = nullptr;        /* the default server behind glint_query_batch */
    std::vector<glint_server *> servers;   /* every live server on this context */
    cudaEvent_t flush_ev[2];
    float last_flush_ms = 0;
    bool last_flushed = false;

    /* active search scratch, allocated on first use */
    uint32_t *d_qbits = nullptr;
    uint32_t *d_qpids = nullptr;
    glint_search_info *d_qout = nullptr;
    unsigned long long *d_qn = nullptr;
    uint64_t qbits_cap = 0, qpids_cap = 0, qout_cap = 0;

    /* misc */
    glint::DevCounters *d_cnt = nullptr;
    glint::DevCounters *h_cnt = nullptr;   /* pinned */
    glint::SinCoef *d_coef = nullptr;
    void *d_scan_tmp = nullptr;
    void *d_scan_tmp_side = nullptr;       /* the schema update's, as it runs beside identify */
    size_t scan_tmp_bytes = 0;
    double2 *h_stage = nullptr;            /* pinned staging for host points (optional) */
    glint::StepParams *h_params = nullptr; /* pinned: the next step's parameters */
    cudaGraph_t graph = nullptr;           /* the captured step (glint_config.use_graph) */
    cudaGraphExec_t graph_exec = nullptr;
    const void *graph_src = nullptr;       /* input buffer the graph copies from */
    glint::StepTimers timers;
    glint_step_stats last_stats;
    bool stats_valid = false;
};

namespace glint {

/* ---- utilities (k_util.cu) ---- */
size_t scan_tmp_bytes(size_t n);
/* exclusive scan of n u32 values into out[0..n], out[n] = total */
cudaError_t scan_u32(const uint32_t *in, uint32_t *out, size_t n, void *tmp, cudaStream_t s);
void init_sin_coef(SinCoef *host);

/* ---- stages ---- */
cudaError_t launch_partition(glint_ctx *c, uint32_t cur_time);
cudaError_t launch_filter(glint_ctx *c);
cudaError_t launch_refine(glint_ctx *c, uint32_t cur_time);
cudaError_t launch_refine_items(glint_ctx *c);
cudaError_t launch_refine_pairs(glint_ctx *c);
struct RefineArgs;
RefineArgs refine_args(glint_ctx *c);
cudaError_t launch_refine_precision_batch(const RefineArgs *d_args, uint32_t R, uint32_t cap_max, uint32_t *ex_off,
                                          uint32_t *wk_off, unsigned int *next, cudaStream_t s);
void launch_step_front(glint_ctx *c, const double *points, bool host);
void launch_step_back(glint_ctx *c);
void begin_step(glint_ctx *c, uint32_t cur_time);
bool device_points(glint_ctx *c, const void *p);
cudaError_t launch_insert(glint_ctx *c, uint32_t cur_time);
cudaError_t launch_identify(glint_ctx *c, uint32_t cur_time);
cudaError_t launch_schema_update(glint_ctx *c, cudaStream_t s, void *scan_tmp);
cudaError_t launch_keys(glint_ctx *c);
cudaError_t flush_alloc(glint_ctx *c);
void flush_free(glint_ctx *c);
void flush_set_attributes();
glint_status run_flush(glint_ctx *c, glint_store_info *info, std::string &err);
void store_blocks_free(glint_ctx *c);
/* CTF::get_ctf_bits + eight_parallel on the host (k_flush.cu) */
bool ctf_bits(glint_ctf_meta &c, const glint_box &map, uint32_t num_objects, uint32_t max_meet_time);
/* stable LSD radix sort of (u64 key, u32 value) pairs (k_sort.cu) */
cudaError_t radix_sort_u64(unsigned long long *keys, uint32_t *vals, unsigned long long *tmp_k, uint32_t *tmp_v,
                           uint64_t n, int bits, void *rs_tmp, void *scan_tmp, cudaStream_t s);
size_t radix_tmp_bytes(uint64_t n);
/* the same, skipping the passes whose digit every key shares (one stream
 * synchronisation) */
cudaError_t radix_sort_u64_varying(unsigned long long *keys, uint32_t *vals, unsigned long long *tmp_k,
                                   uint32_t *tmp_v, uint64_t n, int bits, void *rs_tmp, void *scan_tmp,
                                   cudaStream_t s);
int radix_bits_for(unsigned long long max_key);
void server_free_default(glint_ctx *c);
void servers_detach(glint_ctx *c);

inline ExactCtx make_exact(glint_ctx *c) {
    ExactCtx e;
    e.r = c->cfg.reach_distance;
    e.dpm_lat = c->dpm_lat;
    e.band = c->band;
    e.coef = c->d_coef;
    e.ambiguous = &c->d_cnt->ambiguous;
    e.rechecks = &c->d_cnt->rechecks;
    return e;
}

inline unsigned int grid_for(uint64_t n, unsigned int block, unsigned int cap = 152u * 32u) {
    uint64_t g = (n + block - 1) / block;
    if (g == 0) g = 1;
    if (g > cap) g = cap;
    return (unsigned int)g;
}

} // namespace glint

#endif
