/*
 * glint_api.cu -- the C ABI (include/glint.h): context lifetime, the
 * per-timestep orchestration, and state readback.
 *
 * glint_create plays cuda_create_device_bench (cuda/geometry.cu:1395-1565):
 * it sizes and allocates device state the way the workbench does
 * (tracing/workbench.cpp:31-47), uploads (or builds) the initial schema, and
 * empties the meeting table.  glint_step plays process_with_gpu
 * (cuda/geometry.cu:1573-2218) for the CPU semantics of the reference's
 * stages: partition -> filter -> refine -> table insert -> identify ->
 * schema update, all enqueued on the context's stream with no host
 * synchronisation between stages.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "glint_internal.cuh"

namespace glint {
void partition_set_attributes();
void refine_set_attributes(uint32_t cap);
void refine_prec_set_attributes(uint32_t cap);
void schema_set_attributes();
size_t refine_smem_bytes(uint32_t cap);
uint64_t identify_tiles(uint64_t B);
cudaError_t noalloc_setup(int device);
/* stamps cover a whole number of identify tiles (the padding stays empty) */
inline uint64_t stamp_bytes(uint64_t B) { return identify_tiles(B) * 8192 + 64; }
/* the new-line bitmap: one bit per 4 slots over the same tiles */
inline uint64_t newline_words(uint64_t B) { return identify_tiles(B) * (8192 / 128); }
} // namespace glint

using namespace glint;

namespace {

constexpr double kPIh = 3.14159265;

/* the reference's degree_per_meter_longitude on the host (util/util.h:59-66);
 * only used for the one-time constants and the initial schema, as the
 * reference's build_schema does (tracing/filter.cpp:30) */
double h_dpm_lon(double lat) {
    double absla = std::fabs(lat);
    if (absla == 90) absla = 89;
    volatile double a = (90 - absla) * kPIh;
    volatile double b = a / 180;
    volatile double s = std::sin(b);
    volatile double t = s * 40076.0;
    volatile double u = t * 1000.0;
    return 360.0 / u;
}

struct HNode {
    double low[2], high[2], mid_x, mid_y;
    int16_t level;
    bool leaf;
    uint32_t leaf_id;
    int child[4];
};

/* QTNode build semantics (index/QTree.h:98-311): a node becomes a branch iff
 * at least grid_capacity objects route to it and width(true)/2 > reach; the
 * concurrent inserts of the reference reach this same tree. */
struct SchemaBuilder {
    const double *pts;
    uint32_t gc;
    double reach;
    std::vector<HNode> nodes;
    std::vector<uint32_t> scratch;

    int make(double lx, double ly, double hx, double hy, int16_t level) {
        HNode n;
        n.low[0] = lx; n.low[1] = ly; n.high[0] = hx; n.high[1] = hy;
        volatile double mx = (hx + lx);
        volatile double my = (hy + ly);
        n.mid_x = mx / 2;
        n.mid_y = my / 2;
        n.level = level;
        n.leaf = true;
        n.leaf_id = 0;
        n.child[0] = n.child[1] = n.child[2] = n.child[3] = -1;
        nodes.push_back(n);
        return (int)nodes.size() - 1;
    }
    void build(int ni, uint32_t *ids, size_t cnt) {
        HNode n = nodes[ni];
        volatile double w = (n.high[0] - n.low[0]);
        double width = w / h_dpm_lon(n.low[1]);
        if (!(cnt >= gc && width / 2 > reach)) return;
        int c0 = make(n.low[0], n.low[1], n.mid_x, n.mid_y, n.level + 1);
        int c1 = make(n.mid_x, n.low[1], n.high[0], n.mid_y, n.level + 1);
        int c2 = make(n.low[0], n.mid_y, n.mid_x, n.high[1], n.level + 1);
        int c3 = make(n.mid_x, n.mid_y, n.high[0], n.high[1], n.level + 1);
        nodes[ni].leaf = false;
        nodes[ni].child[0] = c0; nodes[ni].child[1] = c1; nodes[ni].child[2] = c2; nodes[ni].child[3] = c3;
        size_t counts[4] = {0, 0, 0, 0};
        for (size_t i = 0; i < cnt; ++i) {
            const double x = pts[2 * (size_t)ids[i]], y = pts[2 * (size_t)ids[i] + 1];
            counts[(y > n.mid_y) * 2 + (x > n.mid_x)]++;
        }
        size_t off[4] = {0, counts[0], counts[0] + counts[1], counts[0] + counts[1] + counts[2]};
        size_t pos[4] = {off[0], off[1], off[2], off[3]};
        uint32_t *tmp = scratch.data();
        for (size_t i = 0; i < cnt; ++i) {
            const double x = pts[2 * (size_t)ids[i]], y = pts[2 * (size_t)ids[i] + 1];
            tmp[pos[(y > n.mid_y) * 2 + (x > n.mid_x)]++] = ids[i];
        }
        std::memcpy(ids, tmp, cnt * sizeof(uint32_t));
        const int ch[4] = {c0, c1, c2, c3};
        for (int k = 0; k < 4; ++k) build(ch[k], ids + off[k], counts[k]);
    }
    void set_ids(int ni, uint32_t &id) {
        if (nodes[ni].leaf) nodes[ni].leaf_id = id++;
        else for (int k = 0; k < 4; ++k) set_ids(nodes[ni].child[k], id);
    }
    void emit(int ni, std::vector<glint_schema_node> &out, uint32_t &offset) {
        uint32_t cur = offset++;
        const HNode &n = nodes[ni];
        glint_schema_node &s = out[cur];
        std::memset(&s, 0, sizeof(s));
        s.mid_x = n.mid_x;
        s.mid_y = n.mid_y;
        s.level = n.level;
        s.grid_id = n.leaf ? n.leaf_id : 0;
        s.type = n.leaf ? 2 : 1;
        s.low[0] = n.low[0]; s.low[1] = n.low[1]; s.high[0] = n.high[0]; s.high[1] = n.high[1];
        if (!n.leaf)
            for (int k = 0; k < 4; ++k) {
                out[cur].children[k] = offset;
                emit(n.child[k], out, offset);
            }
    }
};

glint_status cuda_fail(glint_ctx *c, cudaError_t e, const char *where) {
    if (c) {
        c->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    }
    return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
}

template <class T>
cudaError_t dalloc(T **p, size_t count) {
    return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
}

__global__ void k_fill_empty(TRec *tab, uint64_t B) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < B; i += (uint64_t)gridDim.x * blockDim.x) {
        TRec r;
        r.w0 = kEmptyW0;
        r.w1 = 0;
        r.mbr[0] = r.mbr[1] = r.mbr[2] = r.mbr[3] = 0;
        tab[i] = r;
    }
}

__global__ void k_iota(uint32_t *a, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

__global__ void k_step_tail(const uint32_t *qstart, uint32_t N, DevCounters *cnt) {
    cnt->cross_checks = qstart[N];
    cnt->total_checks = N + qstart[N];
}

void free_all(glint_ctx *c) {
    void *ptrs[] = {c->d_pts, c->d_sipos, c->d_sfpos, c->d_sc, c->d_fpos, c->d_ibox, c->d_obj_gid, c->d_obj_lv, c->d_obj_leaf, c->d_order, c->d_grid_count,
                    c->d_grid_start, c->d_grid_cursor, c->d_sorted, c->d_rank_of, c->d_sxy, c->d_sL, c->d_leaf_work,
                    c->d_nodes, c->d_low, c->d_sstack, c->d_gstack, c->d_split, c->d_evscan, c->d_cand, c->d_newgid,
                    c->d_events, c->d_evpos, c->d_evlist, c->d_evdata, c->d_evlevel, c->d_big, c->d_qcount,
                    c->d_qstart, c->d_qlist, c->d_qtmp, c->d_tcount, c->d_tstart, c->d_tcursor, c->d_tlist, c->d_tab,
                    c->d_stamp, c->d_newline, c->d_new, c->d_rextra, c->d_tile_cnt, c->d_tile_off, c->d_log, c->d_cnt, c->d_coef,
                    c->d_scan_tmp, c->d_scan_tmp_side, c->d_qbits, c->d_qpids, c->d_qout, c->d_qn};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    flush_free(c);
    store_blocks_free(c);
    if (c->compact_pool) {
        if (c->stream) cudaStreamSynchronize(c->stream);
        cudaMemPoolDestroy(c->compact_pool);
    }
    server_free_default(c);
    servers_detach(c);
    if (c->h_cnt) cudaFreeHost(c->h_cnt);
    if (c->h_params) cudaFreeHost(c->h_params);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    if (c->timers.created) {
        for (auto &e : c->timers.ev) cudaEventDestroy(e);
        for (auto &e : c->flush_ev) cudaEventDestroy(e);
    }
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->join_ev) cudaEventDestroy(c->join_ev);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
}

/* the fixed-point frame: origin at the low corner of the map (widened to the
 * root node's box), S = 2^k with the wider side spanning [2^39, 2^40) units */
Frame make_frame(const glint_box &mbr, const glint_schema_node &root, double r, double dpm_lat) {
    const double lx = std::min(mbr.low[0], root.low[0]), ly = std::min(mbr.low[1], root.low[1]);
    const double hx = std::max(mbr.high[0], root.high[0]), hy = std::max(mbr.high[1], root.high[1]);
    double ext = std::max(hx - lx, hy - ly);
    if (!(ext > 0) || !std::isfinite(ext)) ext = 1.0;
    int e = 0;
    std::frexp(ext, &e); /* ext < 2^e */
    const int k = std::min(48, std::max(0, 40 - e));
    Frame f;
    f.ox = std::isfinite(lx) ? lx : 0.0;
    f.oy = std::isfinite(ly) ? ly : 0.0;
    f.S = std::ldexp(1.0, k);
    f.kdeg = (float)(kPIh / 180.0);
    f.kc = (float)(40076000.0 / (360.0 * f.S));
    f.cy = (float)(1.0 / (dpm_lat * f.S));
    f.r2 = (float)(r * r);
    f.band0 = (float)(64.0 * std::ldexp(1.0, -24) * r * r);
    f.band1 = (float)(4.0 * r);
    return f;
}

void to_device_nodes(const glint_schema_node *in, uint32_t n, const Frame &f, std::vector<DNode> &dn,
                     std::vector<double2> &lo, std::vector<IBox> &ib) {
    for (uint32_t i = 0; i < n; ++i) {
        DNode d;
        std::memset(&d, 0, sizeof(d));
        d.kmx = dkey(in[i].mid_x);
        d.kmy = dkey(in[i].mid_y);
        d.khx = dkey(in[i].high[0]);
        d.khy = dkey(in[i].high[1]);
        ib[i] = fx_box(in[i].low[0], in[i].low[1], in[i].high[0], in[i].high[1], f);
        for (int k = 0; k < 4; ++k) d.child[k] = in[i].children[k];
        d.gid = in[i].grid_id;
        d.type = (uint8_t)in[i].type;
        d.level = in[i].level;
        d.of = in[i].overflow_count;
        d.uf = in[i].underflow_count;
        dn[i] = d;
        lo[i] = make_double2(in[i].low[0], in[i].low[1]);
    }
}

} // namespace

extern "C" {

int glint_abi_version(void) { return GLINT_ABI_VERSION; }

void glint_struct_sizes(uint32_t out[6]) {
    out[0] = sizeof(glint_config);
    out[1] = sizeof(glint_box);
    out[2] = sizeof(glint_schema_node);
    out[3] = sizeof(glint_schema_init);
    out[4] = sizeof(glint_meeting);
    out[5] = sizeof(glint_step_stats);
}

const char *glint_status_string(glint_status s) {
    switch (s) {
    case GLINT_OK: return "ok";
    case GLINT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GLINT_ERR_CUDA: return "CUDA error";
    case GLINT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GLINT_ERR_CAPACITY: return "device buffer capacity exceeded";
    case GLINT_ERR_UNSUPPORTED: return "unsupported configuration";
    case GLINT_ERR_STATE: return "invalid context state";
    case GLINT_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

void glint_config_defaults(glint_config *cfg, uint32_t n) {
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->num_objects = n;
    cfg->grid_capacity = 50;
    cfg->grid_amplify = 2;
    cfg->num_meeting_buckets = 2ull * n;
    cfg->reach_distance = 2;
    cfg->min_meet_time = 5;
    cfg->max_meet_time = 4096;
    cfg->schema_update_delay = 1;
    cfg->dynamic_schema = 1;
    cfg->phased_lookup = 1;
    cfg->G_bytes = 2;
    cfg->CTF_count = 100;
    cfg->dProbFalse = 100;
    cfg->precision_mode = 0;
    cfg->split_num = 10;
    cfg->store_keep = 16;
}

glint_status glint_create(const glint_config *cfg_in, const glint_box *mbr, const double *first_points,
                          const glint_schema_init *init, glint_ctx **out) {
    if (!cfg_in || !mbr || !out) return GLINT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    glint_config cfg = *cfg_in;
    if (cfg.num_objects == 0 || cfg.grid_capacity == 0 || cfg.reach_distance <= 0 || cfg.refine_chunk > 65536)
        return GLINT_ERR_INVALID_ARGUMENT;
    if (cfg.num_objects >= (1u << 26)) return GLINT_ERR_UNSUPPORTED;   /* OID_BIT = 26, util/util.h:49 */
    if (!cfg.phased_lookup) return GLINT_ERR_UNSUPPORTED;
    if (!init && !first_points) return GLINT_ERR_INVALID_ARGUMENT;
    if (cfg.num_meeting_buckets == 0) cfg.num_meeting_buckets = 2ull * cfg.num_objects;
    if (cfg.schema_update_delay == 0) cfg.schema_update_delay = 1;
    if (cfg.CTF_count == 0) cfg.CTF_count = 100;
    if (cfg.split_num == 0) cfg.split_num = 10;
    if (cfg.G_bytes == 0) cfg.G_bytes = 2;
    if (cfg.max_meet_time == 0) cfg.max_meet_time = 4096;
    /* make_sid numbers split_num^2 cells: one CTF each */
    if (cfg.CTF_count != cfg.split_num * cfg.split_num || cfg.split_num > 64) return GLINT_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GLINT_ERR_NO_DEVICE;
    if ((int)cfg.device >= ndev) return GLINT_ERR_INVALID_ARGUMENT;

    glint_ctx *c = new glint_ctx();
    c->cfg = cfg;
    c->mbr = *mbr;
    c->device = (int)cfg.device;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        /* the highest priority: the schema update's one-block stack replay
         * needs 160 KB of shared memory on one SM, which identify's many
         * short blocks would otherwise keep taking first */
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        e = cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, greatest);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        glint_status st = cuda_fail(c, e, "stream");
        if (c->fork_ev) cudaEventDestroy(c->fork_ev);
        if (c->side) cudaStreamDestroy(c->side);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return st;
    }

    /* sizes, tracing/workbench.cpp:36-47 */
    const uint32_t N = cfg.num_objects;
    c->N = N;
    c->cap = (uint32_t)(cfg.grid_amplify * cfg.grid_capacity);
    c->chunk = cfg.refine_chunk ? cfg.refine_chunk : kCrossChunk;
    const uint32_t per = N / cfg.grid_capacity;
    c->G = 4 * std::max<uint32_t>(100000u, per);
    c->S = (uint32_t)(1.6 * c->G);
    c->B = cfg.num_meeting_buckets;
    c->Bm = ~0ull / c->B;
    c->check_cap = cfg.check_capacity ? cfg.check_capacity : (uint64_t)4 * N + 1024;
    /* on the first step every contact is new: up to ~26 per object in the
     * densest synthetic workloads (measured 26 at 10M objects) */
    c->new_cap = cfg.new_capacity ? cfg.new_capacity : std::max<uint64_t>((uint64_t)40 * N, 1u << 20);
    const uint64_t kv_restriction = (uint64_t)(cfg.G_bytes ? cfg.G_bytes : 2) * 33554432ull; /* config.h:80 */
    c->log_cap = cfg.meeting_log_capacity ? cfg.meeting_log_capacity
                                          : std::max<uint64_t>((uint64_t)N, kv_restriction / 2 + 1000000);
    c->dpm_lat = 360.0 / (40076.0 * 1000.0);
    c->x_buffer = cfg.x_buffer != 0 ? cfg.x_buffer : cfg.reach_distance * h_dpm_lon(mbr->low[1]);
    c->y_buffer = cfg.y_buffer != 0 ? cfg.y_buffer : cfg.reach_distance * c->dpm_lat;
    /* key-value store sizes (util/config.h:77-85) and the first window */
    c->kv_restriction = cfg.kv_restriction ? cfg.kv_restriction : (uint64_t)cfg.G_bytes * 33554432ull;
    /* the reference adds 1e6 keys of headroom (util/config.h:81), which one
     * step of 10M objects (~13M keys) overruns: allow 4 keys per object */
    c->kv_cap = cfg.kv_capacity ? cfg.kv_capacity
                                : c->kv_restriction + std::max<uint64_t>(1000000, 4ull * cfg.num_objects);
    c->end_time_min = cfg.start_time + cfg.min_meet_time; /* tracing/process.cpp:404 */
    /* decisions within 2^-38 relative of the threshold are re-taken exactly */
    c->band = cfg.reach_distance * std::ldexp(1.0, -38);
    if (c->cap == 0 || c->cap > 4096) { delete c; return GLINT_ERR_UNSUPPORTED; }

    const uint32_t G = c->G, S = c->S;
    c->n_tiles = identify_tiles(c->B);
    /* scans: objects, grids, slots, identify tiles and radix-sort digit tables */
    const size_t radix_n = 256 * (((size_t)N + 1023) / 1024) + 1;
    const size_t scan_n = std::max<size_t>({(size_t)N, (size_t)G, (size_t)S, (size_t)c->n_tiles, radix_n}) + 1;
    c->scan_tmp_bytes = scan_tmp_bytes(scan_n);
#define ALLOC(ptr, count)                                                  \
    do {                                                                   \
        cudaError_t _e = dalloc(&(ptr), (count));                          \
        if (_e != cudaSuccess) {                                           \
            glint_status _st = cuda_fail(c, _e, "cudaMalloc " #ptr);       \
            free_all(c);                                                   \
            std::string msg = c->last_error;                               \
            delete c;                                                      \
            (void)msg;                                                     \
            return _st;                                                    \
        }                                                                  \
    } while (0)
    ALLOC(c->d_pts, N);
    ALLOC(c->d_sipos, N);
    ALLOC(c->d_sfpos, N);
    ALLOC(c->d_sc, N);
    ALLOC(c->d_fpos, N);
    ALLOC(c->d_obj_gid, N);
    ALLOC(c->d_obj_lv, N);
    ALLOC(c->d_obj_leaf, N);
    ALLOC(c->d_order, N);
    ALLOC(c->d_grid_count, (size_t)G + 1);
    ALLOC(c->d_grid_start, (size_t)G + 1);
    ALLOC(c->d_grid_cursor, G);
    ALLOC(c->d_sorted, N);
    ALLOC(c->d_rank_of, N);
    ALLOC(c->d_sxy, N);
    ALLOC(c->d_sL, N);
    ALLOC(c->d_leaf_work, G);
    ALLOC(c->d_big, G);
    ALLOC(c->d_nodes, S);
    ALLOC(c->d_low, S);
    ALLOC(c->d_ibox, S);
    ALLOC(c->d_sstack, S);
    ALLOC(c->d_gstack, G);
    ALLOC(c->d_split, (size_t)S + 4);
    ALLOC(c->d_evscan, S);
    ALLOC(c->d_cand, S);
    ALLOC(c->d_newgid, S);
    ALLOC(c->d_events, (size_t)S + 1);
    ALLOC(c->d_evpos, (size_t)S + 1);
    ALLOC(c->d_evlist, S);
    ALLOC(c->d_evdata, 2 * (size_t)S);
    ALLOC(c->d_evlevel, S);
    ALLOC(c->d_qcount, (size_t)N + 1);
    ALLOC(c->d_qstart, (size_t)N + 1);
    ALLOC(c->d_qlist, c->check_cap);
    ALLOC(c->d_qtmp, (size_t)N * 8);
    ALLOC(c->d_tcount, (size_t)G + 1);
    ALLOC(c->d_tstart, (size_t)G + 1);
    ALLOC(c->d_tcursor, G);
    ALLOC(c->d_tlist, c->check_cap);
    ALLOC(c->d_tab, c->B);
    ALLOC(c->d_stamp, stamp_bytes(c->B));
    ALLOC(c->d_newline, newline_words(c->B));
    ALLOC(c->d_new, c->new_cap);
    /* each extra refine item is a further `chunk` checks of one leaf */
    c->rextra_cap = c->check_cap / c->chunk + 1;
    ALLOC(c->d_rextra, c->rextra_cap);
    ALLOC(c->d_tile_cnt, c->n_tiles + 1);
    ALLOC(c->d_tile_off, c->n_tiles + 1);
    ALLOC(c->d_log, c->log_cap);
    ALLOC(c->d_cnt, 1);
    ALLOC(c->d_coef, 1);
    {
        uint8_t *tmp = nullptr;
        ALLOC(tmp, c->scan_tmp_bytes);
        c->d_scan_tmp = tmp;
        uint8_t *tmp2 = nullptr;
        ALLOC(tmp2, c->scan_tmp_bytes);
        c->d_scan_tmp_side = tmp2;
    }
#undef ALLOC
    if ((e = flush_alloc(c)) != cudaSuccess) {
        glint_status st = cuda_fail(c, e, "key-value store");
        free_all(c);
        delete c;
        return st;
    }
    if ((e = cudaMallocHost((void **)&c->h_params, sizeof(StepParams))) != cudaSuccess) {
        glint_status st = cuda_fail(c, e, "cudaMallocHost");
        free_all(c);
        delete c;
        return st;
    }
    std::memset(c->h_params, 0, sizeof(StepParams));
    if ((e = cudaMallocHost((void **)&c->h_cnt, sizeof(DevCounters))) != cudaSuccess) {
        glint_status st = cuda_fail(c, e, "cudaMallocHost");
        free_all(c);
        delete c;
        return st;
    }

    /* initial schema */
    std::vector<glint_schema_node> sch;
    uint32_t ssi = 0, gsi = 0;
    std::vector<uint32_t> sstack(S), gstack(G);
    if (init) {
        if (!init->nodes || init->num_nodes == 0 || init->num_nodes > S || init->schema_stack_index > S ||
            init->grids_stack_index > G) {
            free_all(c);
            delete c;
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        sch.assign(S, glint_schema_node{});
        std::memcpy(sch.data(), init->nodes, sizeof(glint_schema_node) * init->num_nodes);
        for (uint32_t i = init->num_nodes; i < S; ++i) sch[i].type = 0;
        ssi = init->schema_stack_index;
        gsi = init->grids_stack_index;
        for (uint32_t i = 0; i < S; ++i) sstack[i] = init->schema_stack && i < init->num_nodes ? init->schema_stack[i] : i;
        for (uint32_t i = 0; i < G; ++i) gstack[i] = init->grids_stack ? init->grids_stack[i] : i;
    } else {
        SchemaBuilder b;
        b.pts = first_points;
        b.gc = cfg.grid_capacity;
        b.reach = cfg.reach_distance;
        b.scratch.resize(N);
        std::vector<uint32_t> ids(N);
        for (uint32_t i = 0; i < N; ++i) ids[i] = i;
        int root = b.make(mbr->low[0], mbr->low[1], mbr->high[0], mbr->high[1], 0);
        b.build(root, ids.data(), N);
        uint32_t leaf_id = 0;
        b.set_ids(root, leaf_id);
        if (b.nodes.size() > S || leaf_id > G) {
            free_all(c);
            delete c;
            return GLINT_ERR_CAPACITY;
        }
        sch.assign(S, glint_schema_node{});
        uint32_t off = 0;
        b.emit(root, sch, off);
        ssi = (uint32_t)b.nodes.size();
        gsi = leaf_id;
        for (uint32_t i = 0; i < S; ++i) sstack[i] = i;
        for (uint32_t i = 0; i < G; ++i) gstack[i] = i;
    }
    if (sch[0].type != 1) {
        /* the reference descends from the root's children (filter.cpp:229-243);
         * a root leaf has none */
        free_all(c);
        delete c;
        return GLINT_ERR_UNSUPPORTED;
    }
    c->frame = make_frame(*mbr, sch[0], cfg.reach_distance, c->dpm_lat);
    std::vector<DNode> dn(S);
    std::vector<double2> lo(S);
    std::vector<IBox> ib(S);
    to_device_nodes(sch.data(), S, c->frame, dn, lo, ib);
    cudaMemcpy(c->d_nodes, dn.data(), sizeof(DNode) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_low, lo.data(), sizeof(double2) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_ibox, ib.data(), sizeof(IBox) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_sstack, sstack.data(), sizeof(uint32_t) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_gstack, gstack.data(), sizeof(uint32_t) * G, cudaMemcpyHostToDevice);
    DevCounters hc;
    std::memset(&hc, 0, sizeof(hc));
    hc.ssi = ssi;
    hc.gsi = gsi;
    cudaMemcpy(c->d_cnt, &hc, sizeof(hc), cudaMemcpyHostToDevice);
    SinCoef coef;
    init_sin_coef(&coef);
    cudaMemcpy(c->d_coef, &coef, sizeof(coef), cudaMemcpyHostToDevice);
    k_fill_empty<<<grid_for(c->B, 256, 152u * 16u), 256, 0, c->stream>>>(c->d_tab, c->B);
    cudaMemsetAsync(c->d_stamp, 0, stamp_bytes(c->B), c->stream);
    cudaMemsetAsync(c->d_newline, 0, sizeof(uint32_t) * newline_words(c->B), c->stream);
    cudaMemsetAsync(c->d_grid_count, 0, sizeof(uint32_t) * ((size_t)G + 1), c->stream);
    k_iota<<<grid_for(N, 256, 152u * 8u), 256, 0, c->stream>>>(c->d_order, N);
    /* scratch address of glint_active_search_noalloc, once per device, with
     * this device current; a failure is reported by that call */
    noalloc_setup(c->device);
    partition_set_attributes();
    refine_set_attributes(c->cap);
    refine_prec_set_attributes(c->cap);
    schema_set_attributes();
    flush_set_attributes();
    for (auto &ev : c->timers.ev) cudaEventCreate(&ev);
    for (auto &ev : c->flush_ev) cudaEventCreate(&ev);
    c->timers.created = true;
    e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        glint_status st = cuda_fail(c, e, "create");
        free_all(c);
        delete c;
        return st;
    }
    *out = c;
    return GLINT_OK;
}

glint_status glint_destroy(glint_ctx *c) {
    if (!c) return GLINT_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return GLINT_OK;
}

const char *glint_last_error(const glint_ctx *c) { return c ? c->last_error.c_str() : "no context"; }

void *glint_stream(glint_ctx *c) { return c ? (void *)c->stream : nullptr; }

glint_status glint_get_capacities(const glint_ctx *c, uint32_t *sc, uint32_t *gc, uint64_t *b) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    if (sc) *sc = c->S;
    if (gc) *gc = c->G;
    if (b) *b = c->B;
    return GLINT_OK;
}

} // extern "C"

namespace glint {

/* The launches of one step, from the counter reset to the copy of the
 * counters to the host; no host synchronisation, so they can be captured.
 * A step is its front (up to the refine stage's work items), the refine
 * pair tests, and its back: a batch of regions runs every front, then one
 * refine launch over all regions, then every back. */
void launch_step_front(glint_ctx *c, const double *points, bool host) {
    cudaStream_t s = c->stream;
    const bool tm = c->cfg.timing != 0 && !c->cfg.use_graph;
    cudaMemsetAsync(c->d_cnt, 0, kStepCounterBytes, s);
    cudaMemcpyAsync(&c->d_cnt->step_time, c->h_params, sizeof(StepParams), cudaMemcpyHostToDevice, s);
    if (tm) cudaEventRecord(c->timers.ev[0], s);
    if (host) {
        cudaMemcpyAsync(c->d_pts, points, sizeof(double2) * c->N, cudaMemcpyHostToDevice, s);
    } else if ((const void *)points != (const void *)c->d_pts) {
        cudaMemcpyAsync(c->d_pts, points, sizeof(double2) * c->N, cudaMemcpyDeviceToDevice, s);
    }
    if (tm) cudaEventRecord(c->timers.ev[1], s);
    launch_partition(c, 0);
    if (tm) cudaEventRecord(c->timers.ev[2], s);
    launch_filter(c);
    if (tm) cudaEventRecord(c->timers.ev[3], s);
    launch_refine_items(c);
}

void launch_step_back(glint_ctx *c) {
    cudaStream_t s = c->stream;
    const bool tm = c->cfg.timing != 0 && !c->cfg.use_graph;
    if (tm) cudaEventRecord(c->timers.ev[4], s);
    launch_insert(c, 0);
    if (tm) cudaEventRecord(c->timers.ev[5], s);
    /* The schema update reads the leaf counts and rewrites the schema and its
     * stacks; identify and the key append use the table, the log and the
     * key buffers.  Neither reads what the other writes, so the update runs
     * on the side stream while identify streams the table. */
    const bool schema = c->cfg.dynamic_schema != 0;
    if (schema) {
        cudaEventRecord(c->fork_ev, s);
        cudaStreamWaitEvent(c->side, c->fork_ev, 0);
        launch_schema_update(c, c->side, c->d_scan_tmp_side);
        cudaEventRecord(c->join_ev, c->side);
    }
    launch_identify(c, 0);
    launch_keys(c);
    if (tm) cudaEventRecord(c->timers.ev[6], s);
    if (schema) cudaStreamWaitEvent(s, c->join_ev, 0);
    k_step_tail<<<1, 1, 0, s>>>(c->d_qstart, c->N, c->d_cnt);
    if (tm) cudaEventRecord(c->timers.ev[7], s);
    cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, s);
}

static void launch_step(glint_ctx *c, const double *points, bool host) {
    launch_step_front(c, points, host);
    launch_refine_pairs(c);
    launch_step_back(c);
}

/* the host side of starting a step: its number, time, tag and the
 * parameters the captured memcpy reads when the step runs */
void begin_step(glint_ctx *c, uint32_t cur_time) {
    c->step_index++;
    c->last_time = cur_time;
    c->h_params->step_time = cur_time;
    c->h_params->step_tag = stamp_of(c->step_index);
    c->h_params->end_time_min = c->end_time_min;
    c->stats_valid = false;
}

/* the step's input must be device (or managed) memory: an address that is
 * neither would reach the copy engine unchecked */
bool device_points(glint_ctx *c, const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        c->last_error = "step input: not a CUDA pointer";
        return false;
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) {
        c->last_error = "step input: not device memory";
        return false;
    }
    return true;
}

} // namespace glint

extern "C" {

static glint_status enqueue_step(glint_ctx *c, const double *points, bool host, uint32_t cur_time,
                                 bool allow_graph = true) {
    cudaStream_t s = c->stream;
    /* a captured step reads its parameters from host memory when it runs:
     * the previous step must have finished before they are overwritten */
    if (c->cfg.use_graph && c->step_index > 0) cudaStreamSynchronize(s);
    begin_step(c, cur_time);
    if (!c->cfg.use_graph || host || !allow_graph) {
        launch_step(c, points, host);
    } else {
        if (c->graph_exec && c->graph_src != (const void *)points) {
            cudaGraphExecDestroy(c->graph_exec);
            cudaGraphDestroy(c->graph);
            c->graph_exec = nullptr;
            c->graph = nullptr;
        }
        if (!c->graph_exec) {
            cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(c, e, "step capture");
            launch_step(c, points, false);
            e = cudaStreamEndCapture(s, &c->graph);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&c->graph_exec, c->graph, 0);
            if (e != cudaSuccess) return cuda_fail(c, e, "step capture");
            c->graph_src = points;
        }
        cudaError_t e = cudaGraphLaunch(c->graph_exec, s);
        if (e != cudaSuccess) return cuda_fail(c, e, "step graph");
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "step launch");
    return GLINT_OK;
}

static void fill_stats(glint_ctx *c, glint_step_stats *st) {
    const DevCounters &h = *c->h_cnt;
    std::memset(st, 0, sizeof(*st));
    st->cur_time = c->last_time;
    st->checks = h.total_checks;
    st->border_objects = h.border_objects;
    st->cross_checks = h.cross_checks;
    st->candidates = h.candidates;
    st->contacts = h.contacts;
    st->new_keys = h.new_keys;
    st->num_taken_buckets = h.taken;
    st->num_active_meetings = h.active;
    st->meetings = h.meetings;
    st->splits = h.splits;
    st->merges = h.merges;
    st->leaves = h.gsi;
    st->nodes = h.ssi;
    st->dropped_objects = h.dropped;
    st->rechecks = h.rechecks;
    st->ambiguous = h.ambiguous;
    st->band_pairs = h.band_pairs;
    st->box_band = h.box_band;
    st->error_flags = h.error_flags;
    /* kernels per step: partition 9, filter 9, refine 2 (work items, pairs),
     * insert 1, identify 6 + keys 1, schema update 11, tail 1 (scans count
     * three each) */
    st->launches = 9 + 9 + 2 + 1 + 7 + (c->cfg.dynamic_schema ? 11 : 0) + 1;
    st->meeting_log_size = h.log_head;
    st->kv_count = h.kv_count;
    st->flushed = c->last_flushed ? 1u : 0u;
    st->flush_ms = c->last_flush_ms;
    if (c->cfg.timing && !c->cfg.use_graph) {
        for (int k = 0; k < 7; ++k) cudaEventElapsedTime(&st->ms[k], c->timers.ev[k], c->timers.ev[k + 1]);
        cudaEventElapsedTime(&st->ms[7], c->timers.ev[0], c->timers.ev[7]);
    }
}

glint_status glint_sync(glint_ctx *c, glint_step_stats *st) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "sync");
    if (!c->stats_valid) {
        c->last_flushed = false;
        c->last_flush_ms = 0;
    }
    if (c->cfg.auto_flush && !c->stats_valid && c->h_cnt->kv_count > c->kv_restriction &&
        !(c->h_cnt->error_flags & GLINT_EF_KV_OVERFLOW)) {
        /* the reference flushes inside the step once kv_count passes
         * kv_restriction (cuda/geometry.cu:1752) */
        cudaEventRecord(c->flush_ev[0], c->stream);
        std::string err;
        const glint_status fs = run_flush(c, nullptr, err);
        cudaEventRecord(c->flush_ev[1], c->stream);
        cudaEventSynchronize(c->flush_ev[1]);
        if (fs != GLINT_OK) {
            c->last_error = err;
            return fs;
        }
        cudaEventElapsedTime(&c->last_flush_ms, c->flush_ev[0], c->flush_ev[1]);
        c->last_flushed = true;
        cudaMemcpy(c->h_cnt, c->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost);
    }
    fill_stats(c, &c->last_stats);
    c->stats_valid = true;
    if (st) *st = c->last_stats;
    if (c->last_stats.error_flags & (GLINT_EF_CHECKS_OVERFLOW | GLINT_EF_NEW_OVERFLOW | GLINT_EF_TABLE_FULL |
                                     GLINT_EF_SCHEMA_STACK | GLINT_EF_SEGMENT_TOO_LARGE | GLINT_EF_DFS_OVERFLOW |
                                     GLINT_EF_DUPLICATE_NEW | GLINT_EF_TREE_DEPTH | GLINT_EF_LOG_OVERFLOW |
                                     GLINT_EF_KV_OVERFLOW | GLINT_EF_STORE_DOMAIN)) {
        char buf[96];
        std::snprintf(buf, sizeof(buf), "capacity or consistency error, flags 0x%x", c->last_stats.error_flags);
        c->last_error = buf;
        return GLINT_ERR_CAPACITY;
    }
    return GLINT_OK;
}

glint_status glint_step_device(glint_ctx *c, const double *d_points, uint32_t cur_time) {
    if (!c || !d_points) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "step")) return GLINT_ERR_STATE;
    cudaSetDevice(c->device);
    if (!device_points(c, d_points)) return GLINT_ERR_INVALID_ARGUMENT;
    return enqueue_step(c, d_points, false, cur_time);
}

glint_status glint_step(glint_ctx *c, const double *points, uint32_t cur_time, glint_step_stats *st) {
    if (!c || !points) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "step")) return GLINT_ERR_STATE;
    cudaSetDevice(c->device);
    glint_status r = enqueue_step(c, points, true, cur_time);
    if (r != GLINT_OK) return r;
    return glint_sync(c, st);
}

glint_status glint_host_alloc(size_t bytes, void **out) {
    if (!out) return GLINT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        *out = nullptr;
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    return GLINT_OK;
}

glint_status glint_host_free(void *p) {
    if (p && cudaFreeHost(p) != cudaSuccess) return GLINT_ERR_CUDA;
    return GLINT_OK;
}

glint_status glint_meetings(glint_ctx *c, glint_meeting *out, uint64_t cap, uint64_t *n) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "meetings")) return GLINT_ERR_STATE;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "meetings");
    const uint64_t total = c->h_cnt->meetings;
    const uint64_t begin = c->h_cnt->log_step_begin;
    if (n) *n = total;
    const uint64_t m = std::min<uint64_t>(std::min<uint64_t>(total, cap), c->log_cap);
    if (!out || m == 0) return GLINT_OK;
    const uint64_t b = begin % c->log_cap;
    const uint64_t first = std::min<uint64_t>(m, c->log_cap - b);
    e = cudaMemcpy(out, c->d_log + b, sizeof(glint_meeting) * first, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && first < m)
        e = cudaMemcpy(out + first, c->d_log, sizeof(glint_meeting) * (m - first), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "meetings copy");
    return GLINT_OK;
}

glint_status glint_get_schema(glint_ctx *c, glint_schema_node *nodes, uint32_t *schema_stack, uint32_t *grids_stack,
                              uint32_t *grid_counter, uint32_t *ssi, uint32_t *gsi) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(c->stream);
    DevCounters h;
    cudaMemcpy(&h, c->d_cnt, sizeof(h), cudaMemcpyDeviceToHost);
    if (ssi) *ssi = h.ssi;
    if (gsi) *gsi = h.gsi;
    if (nodes) {
        std::vector<DNode> dn(c->S);
        std::vector<double2> lo(c->S);
        cudaMemcpy(dn.data(), c->d_nodes, sizeof(DNode) * c->S, cudaMemcpyDeviceToHost);
        cudaMemcpy(lo.data(), c->d_low, sizeof(double2) * c->S, cudaMemcpyDeviceToHost);
        for (uint32_t i = 0; i < c->S; ++i) {
            glint_schema_node &s = nodes[i];
            std::memset(&s, 0, sizeof(s));
            s.grid_id = dn[i].gid;
            s.level = dn[i].level;
            s.type = dn[i].type;
            s.overflow_count = dn[i].of;
            s.underflow_count = dn[i].uf;
            s.mid_x = kdbl(dn[i].kmx);
            s.mid_y = kdbl(dn[i].kmy);
            s.low[0] = lo[i].x;
            s.low[1] = lo[i].y;
            s.high[0] = kdbl(dn[i].khx);
            s.high[1] = kdbl(dn[i].khy);
            for (int k = 0; k < 4; ++k) s.children[k] = dn[i].child[k];
        }
    }
    if (schema_stack) cudaMemcpy(schema_stack, c->d_sstack, sizeof(uint32_t) * c->S, cudaMemcpyDeviceToHost);
    if (grids_stack) cudaMemcpy(grids_stack, c->d_gstack, sizeof(uint32_t) * c->G, cudaMemcpyDeviceToHost);
    if (grid_counter) cudaMemcpy(grid_counter, c->d_grid_count, sizeof(uint32_t) * c->G, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GLINT_OK : cuda_fail(c, e, "get_schema");
}

glint_status glint_get_buckets(glint_ctx *c, uint64_t *keys, uint32_t *starts, float *mbrs) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "buckets")) return GLINT_ERR_STATE;
    cudaStreamSynchronize(c->stream);
    const uint64_t chunk = 1ull << 22;
    std::vector<TRec> buf((size_t)std::min<uint64_t>(chunk, c->B));
    for (uint64_t b = 0; b < c->B; b += chunk) {
        const uint64_t n = std::min<uint64_t>(chunk, c->B - b);
        cudaMemcpy(buf.data(), c->d_tab + b, sizeof(TRec) * n, cudaMemcpyDeviceToHost);
        for (uint64_t i = 0; i < n; ++i) {
            const unsigned long long w0 = buf[i].w0;
            if (keys) keys[b + i] = (w0 == kEmptyW0) ? kEmptyKey : cantor(pair_a(w0), pair_b(w0));
            if (starts) starts[b + i] = (uint32_t)buf[i].w1;
            if (mbrs)
                for (int k = 0; k < 4; ++k) mbrs[4 * (b + i) + k] = fdec(buf[i].mbr[k]);
        }
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GLINT_OK : cuda_fail(c, e, "get_buckets");
}

} /* extern "C" */

namespace glint {
/* the step on device points, never through the captured graph (whose input
 * buffer is fixed) */
glint_status enqueue_device_step_plain(glint_ctx *c, const double *d_points, uint32_t cur_time) {
    return enqueue_step(c, d_points, false, cur_time, false);
}
} // namespace glint
