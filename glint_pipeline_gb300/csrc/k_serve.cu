/*
 * k_serve.cu -- contact-trace queries over the flushed store, served with
 * continuous batching.
 *
 * Reference: id_search_in_CTB / id_search_in_disk (tracing/workbench.cpp:
 * 397-444) read one object's keys per call: its sid picks a CTF (or the
 * oversize buffer, sid 1), CTF::binary_search / oversize_buffer::
 * search_buffer find its first key and the walk of search_SSTable visits the
 * rest (tracing/step_merge.cpp:67-115, 501-568); the targets of one hop are
 * the search list of the next (search_multi_pid, tracing/process.cpp:476-495).
 *
 * Device form: every query owns a slot, a visited bitmap over objects and
 * two object lists (frontier, next).  One launch advances every active slot
 * by one hop: its items are (slot, frontier object, kept block) triples,
 * over the kept blocks whose time span can meet the slot's window; the
 * object's sid, first and count in the block locate its keys, which are
 * decoded as CTF::parse_key does (tracing/step_merge.cpp:335-345), and each
 * target inside the time window that the slot has not visited joins its next
 * list.  Between launches the host retires finished queries and admits
 * waiting ones into free slots (continuous batching); a slot's result only
 * depends on its own query.
 */
#include <algorithm>
#include <cstring>
#include <deque>
#include <unordered_map>
#include <vector>

#include "glint_internal.cuh"
#include "store_codec.cuh"

namespace glint {

constexpr uint32_t kMaxHops = 8;

struct SlotParam {
    uint32_t t_start, t_end, window, cur;  /* cur: which list holds the frontier */
};

struct HopArgs {
    const StoreBlockDev *blocks;
    uint32_t nblocks;
    uint32_t N;
    uint64_t words;                        /* bitmap words per slot */
    uint32_t *visited;                     /* [slot][words] */
    uint32_t *lists;                       /* [slot][2][N] */
    const SlotParam *param;                /* [slot] */
    uint32_t *counts;                      /* [slot] next-list sizes */
    unsigned long long *scanned;           /* [slot] keys read */
    const uint32_t *active;                /* [A] slots taking part in this launch */
    const unsigned long long *prefix;      /* [A + 1] their items (frontier x blocks), prefix sums */
    const uint32_t *rel;                   /* each active slot's blocks, concatenated */
    const uint32_t *rel_off;               /* [A + 1] where each active slot's blocks start in rel */
    uint32_t A;
};

/* marks target reached for slot s and appends it to the slot's next list
 * when it is new; the lanes that call together and append to the same slot
 * take their places with one atomic (a slot's counter is one address that
 * every new object of a large frontier would otherwise hit) */
__device__ inline void visit(const HopArgs &a, uint32_t s, uint32_t next_list, uint32_t target) {
    const unsigned calling = __activemask();
    bool fresh = false;
    if (target < a.N) {
        /* a query's bits only go from 0 to 1, so a set bit read from L2 is
         * final and saves the atomic; a clear one is settled by the atomic */
        const uint32_t bit = 1u << (target & 31);
        uint32_t *w = &a.visited[(size_t)s * a.words + (target >> 5)];
        if (!(__ldcg(w) & bit)) fresh = !(atomicOr(w, bit) & bit);
    }
    const unsigned appending = __ballot_sync(calling, fresh);
    if (!fresh) return;
    const unsigned peers = __match_any_sync(appending, s);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&a.counts[s], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const uint32_t idx = base + __popc(peers & ((1u << lane) - 1u));
    if (idx < a.N) a.lists[((size_t)s * 2 + next_list) * a.N + idx] = target;
}

__global__ void __launch_bounds__(256) k_serve_hop(HopArgs a) {
    const unsigned long long total = a.prefix[a.A];
    /* keys read, per slot: summed here while this thread's items stay in one
     * slot (slots own contiguous item ranges), added once when they move on */
    uint32_t acc_slot = 0xffffffffu;
    unsigned long long acc = 0;
    for (unsigned long long it = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; it < total;
         it += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = a.A; /* prefix[lo] <= it < prefix[lo + 1] */
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (a.prefix[mid] <= it) lo = mid;
            else hi = mid;
        }
        /* block-major within a slot: consecutive items take consecutive
         * frontier objects (ascending ids) of one block, whose sids,
         * key ranges and keys then lie close together */
        const uint32_t nrel = a.rel_off[lo + 1] - a.rel_off[lo];
        const unsigned long long fr = (a.prefix[lo + 1] - a.prefix[lo]) / nrel;
        const unsigned long long local = it - a.prefix[lo];
        const unsigned long long bi = local / fr;
        const unsigned long long f = local - bi * fr;
        const uint32_t b = a.rel[a.rel_off[lo] + (uint32_t)bi];
        const uint32_t s = a.active[lo];
        const SlotParam sp = a.param[s];
        const uint32_t obj = a.lists[((size_t)s * 2 + sp.cur) * a.N + f];
        const StoreBlockDev blk = a.blocks[b];
        const uint32_t sid = blk.sids[obj];
        if (sid == 0) continue;
        const uint32_t n = blk.count[obj], first = blk.first[obj];
        const uint32_t nl = sp.cur ^ 1u;
        if (s != acc_slot) {
            if (acc) atomicAdd(&a.scanned[acc_slot], acc);
            acc_slot = s;
            acc = 0;
        }
        acc += n;
        if (sid == 1) {
            for (uint32_t j = 0; j < n; ++j) {
                const ulonglong2 k = blk.okeys[first + j];
                const uint32_t end = (uint32_t)k.x + blk.end_time_min, duration = (uint32_t)(k.x >> 32);
                const uint32_t start = end - duration;
                if (sp.window && !(start < sp.t_end && sp.t_start < end)) continue;
                visit(a, s, nl, (uint32_t)k.y & ((1u << 26) - 1));
            }
            continue;
        }
        const uint32_t c = sid - 2;
        if (c >= blk.C) continue;
        const glint_ctf_meta m = blk.ctfs[c];
        const uint32_t kb = m.key_bit / 8;
        const uint8_t *base = blk.keys + blk.byte_index[c] + (unsigned long long)(first - blk.key_index[c]) * kb;
        for (uint32_t j = 0; j < n; ++j) {
            const uint8_t *p = base + (size_t)j * kb;
            unsigned __int128 v = load_key(p, kb, blk.keys + blk.key_bytes);
            v >>= m.mbr_bit;
            const uint32_t end = (uint32_t)(v & ((1ull << m.end_bit) - 1)) + blk.end_time_min;
            v >>= m.end_bit;
            const uint32_t duration = (uint32_t)(v & ((1ull << m.duration_bit) - 1));
            v >>= m.duration_bit;
            const uint32_t target = (uint32_t)(v & ((1ull << m.id_bit) - 1));
            const uint32_t start = end - duration;
            if (sp.window && !(start < sp.t_end && sp.t_start < end)) continue;
            visit(a, s, nl, target);
        }
    }
    if (acc) atomicAdd(&a.scanned[acc_slot], acc);
}

/* the new ids of the active slots as (slot rank, id) keys: slot rank r's
 * count[r] ids start at off[r] */
__global__ void k_serve_collect(const uint32_t *__restrict__ lists, uint32_t N, const uint32_t *__restrict__ act,
                                const SlotParam *__restrict__ param, const unsigned long long *__restrict__ off,
                                uint32_t A, unsigned long long *__restrict__ keys, uint32_t *__restrict__ vals) {
    const unsigned long long total = off[A];
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = A; /* off[lo] <= i < off[lo + 1] */
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (off[mid] <= i) lo = mid;
            else hi = mid;
        }
        const uint32_t s = act[lo];
        const uint32_t id = lists[((size_t)s * 2 + param[s].cur) * N + (i - off[lo])];
        keys[i] = ((unsigned long long)lo << 32) | id;
        vals[i] = 0;
    }
}

__global__ void k_serve_ids(const unsigned long long *__restrict__ keys, uint64_t n, uint32_t *__restrict__ ids) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        ids[i] = (uint32_t)keys[i];
}

/* the seeds of newly admitted slots: visited, and listed as their frontier */
__global__ void k_serve_seed(const uint32_t *__restrict__ seeds, const unsigned long long *__restrict__ sprefix,
                             const uint32_t *__restrict__ slots, uint32_t n_slots, HopArgs a) {
    const unsigned long long total = sprefix[n_slots];
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_slots;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (sprefix[mid] <= i) lo = mid;
            else hi = mid;
        }
        const uint32_t s = slots[lo];
        const uint32_t p = seeds[i];
        if (p >= a.N) continue;
        uint32_t *vis = a.visited + (size_t)s * a.words;
        const uint32_t bit = 1u << (p & 31);
        if (atomicOr(&vis[p >> 5], bit) & bit) continue;
        const uint32_t idx = atomicAdd(&a.counts[s], 1u);
        a.lists[((size_t)s * 2 + a.param[s].cur) * a.N + idx] = p;
    }
}

} // namespace glint

using namespace glint;

struct PendingQuery {
    uint64_t ticket;
    std::vector<uint32_t> seeds;
    uint32_t hops, t_start, t_end;
};

struct SlotState {
    bool busy = false;
    uint64_t ticket = 0;
    uint32_t hops = 0, hop = 0, cur = 0, frontier = 0;
    std::vector<uint32_t> ids;
    uint64_t hop_end[kMaxHops] = {};
};

struct FinishedQuery {
    std::vector<uint32_t> ids;
    uint64_t hop_end[kMaxHops];
    uint64_t keys_scanned;
};

struct glint_server {
    glint_ctx *ctx = nullptr;
    uint32_t slots = 0;
    uint64_t words = 0;
    uint32_t *visited = nullptr, *lists = nullptr, *counts = nullptr, *active = nullptr, *seed_slots = nullptr;
    SlotParam *param = nullptr;
    unsigned long long *scanned = nullptr, *prefix = nullptr, *sprefix = nullptr;
    uint32_t *seeds = nullptr;
    uint64_t seeds_cap = 0;
    StoreBlockDev *blocks = nullptr;
    uint32_t blocks_cap = 0;
    uint32_t *rel = nullptr, *rel_off = nullptr;   /* each active slot's blocks (the window's) */
    uint64_t rel_cap = 0, rel_off_cap = 0;
    uint64_t next_ticket = 1;
    std::deque<PendingQuery> queue;
    std::vector<SlotState> state;
    std::vector<SlotParam> hparam;
    std::unordered_map<uint64_t, FinishedQuery> done;
    std::vector<uint32_t> buf;
    /* a hop's new ids of all active slots, sorted by (slot, id) on the device */
    unsigned long long *rk = nullptr, *rk2 = nullptr, *roff = nullptr;
    uint32_t *rv = nullptr, *rv2 = nullptr, *rids = nullptr;
    void *rs_tmp = nullptr, *rscan = nullptr;
    uint64_t r_cap = 0;
};

static void server_release(glint_server *v) {
    void *ps[] = {v->visited, v->lists, v->counts, v->active, v->seed_slots, v->param, v->scanned, v->prefix,
                  v->sprefix, v->seeds, v->blocks, v->rk, v->rk2, v->roff, v->rv, v->rv2, v->rids, v->rs_tmp,
                  v->rscan, v->rel, v->rel_off};
    for (void *p : ps)
        if (p) cudaFree(p);
}

/* the results' sort buffers for n ids over `act` slots (grown, never shrunk) */
static cudaError_t server_result_space(glint_server *v, uint64_t n, uint32_t act) {
    if (n <= v->r_cap && v->roff) return cudaSuccess;
    const uint64_t cap = std::max<uint64_t>(n, 1u << 20);
    void *ps[] = {v->rk, v->rk2, v->rv, v->rv2, v->rids, v->rs_tmp, v->rscan};
    for (void *p : ps)
        if (p) cudaFree(p);
    v->rk = v->rk2 = nullptr;
    v->rv = v->rv2 = v->rids = nullptr;
    v->rs_tmp = v->rscan = nullptr;
    v->r_cap = 0;
    cudaError_t e = cudaMalloc((void **)&v->rk, sizeof(unsigned long long) * cap);
    if (e == cudaSuccess) e = cudaMalloc((void **)&v->rk2, sizeof(unsigned long long) * cap);
    if (e == cudaSuccess) e = cudaMalloc((void **)&v->rv, sizeof(uint32_t) * cap);
    if (e == cudaSuccess) e = cudaMalloc((void **)&v->rv2, sizeof(uint32_t) * cap);
    if (e == cudaSuccess) e = cudaMalloc((void **)&v->rids, sizeof(uint32_t) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&v->rs_tmp, radix_tmp_bytes(cap));
    if (e == cudaSuccess) e = cudaMalloc(&v->rscan, scan_tmp_bytes(256 * ((cap + 1023) / 1024) + 1));
    if (e == cudaSuccess && !v->roff) e = cudaMalloc((void **)&v->roff, sizeof(unsigned long long) * (v->slots + 1));
    if (e == cudaSuccess) v->r_cap = cap;
    (void)act;
    return e;
}

extern "C" glint_status glint_server_create(glint_ctx *c, uint32_t max_slots, glint_server **out) {
    if (!c || !out || max_slots == 0) return GLINT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cudaSetDevice(c->device);
    glint_server *v = new glint_server();
    v->ctx = c;
    v->words = ((uint64_t)c->N + 31) / 32;
    /* admission by memory: a slot costs its bitmap and two lists */
    const size_t slot_bytes = sizeof(uint32_t) * (v->words + 2 * (size_t)c->N) + 64;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t fit = (free_b / 2) / slot_bytes;
    v->slots = (uint32_t)std::min<size_t>(max_slots, std::max<size_t>(fit, 1));
    const uint32_t S = v->slots;
    cudaError_t e = cudaSuccess;
    auto A = [&](void **p, size_t n) {
        if (e == cudaSuccess) e = cudaMalloc(p, n ? n : 1);
    };
    A((void **)&v->visited, sizeof(uint32_t) * v->words * S);
    A((void **)&v->lists, sizeof(uint32_t) * 2 * (size_t)c->N * S);
    A((void **)&v->counts, sizeof(uint32_t) * S);
    A((void **)&v->active, sizeof(uint32_t) * S);
    A((void **)&v->seed_slots, sizeof(uint32_t) * S);
    A((void **)&v->param, sizeof(SlotParam) * S);
    A((void **)&v->scanned, sizeof(unsigned long long) * S);
    A((void **)&v->prefix, sizeof(unsigned long long) * (S + 1));
    A((void **)&v->sprefix, sizeof(unsigned long long) * (S + 1));
    if (e != cudaSuccess) {
        server_release(v);
        delete v;
        c->last_error = std::string("server: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    v->state.resize(S);
    v->hparam.resize(S);
    c->servers.push_back(v);
    *out = v;
    return GLINT_OK;
}

/* a server whose context was destroyed first is detached: its device memory
 * is released with the context and only the handle remains */
extern "C" glint_status glint_server_destroy(glint_server *v) {
    if (!v) return GLINT_OK;
    if (v->ctx) {
        glint_ctx *c = v->ctx;
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->stream);
        server_release(v);
        c->servers.erase(std::remove(c->servers.begin(), c->servers.end(), v), c->servers.end());
        if (c->server == v) c->server = nullptr;
    }
    delete v;
    return GLINT_OK;
}

extern "C" uint32_t glint_server_slots(const glint_server *v) { return v ? v->slots : 0u; }

extern "C" glint_status glint_server_submit(glint_server *v, const glint_query *q, uint64_t *ticket) {
    if (v && !v->ctx) return GLINT_ERR_STATE;
    if (!v || !q || (q->n_seeds && !q->seeds) || q->hops == 0 || q->hops > kMaxHops) return GLINT_ERR_INVALID_ARGUMENT;
    PendingQuery p;
    p.ticket = v->next_ticket++;
    p.seeds.assign(q->seeds, q->seeds + q->n_seeds);
    p.hops = q->hops;
    p.t_start = q->t_start;
    p.t_end = q->t_end;
    v->queue.push_back(std::move(p));
    if (ticket) *ticket = v->queue.back().ticket;
    return GLINT_OK;
}

static glint_status server_fail(glint_server *v, cudaError_t e, const char *where) {
    v->ctx->last_error = std::string("server ") + where + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
}

static HopArgs server_args(glint_server *v, uint32_t nb) {
    HopArgs a;
    a.blocks = v->blocks;
    a.nblocks = nb;
    a.N = v->ctx->N;
    a.words = v->words;
    a.visited = v->visited;
    a.lists = v->lists;
    a.param = v->param;
    a.counts = v->counts;
    a.scanned = v->scanned;
    a.active = v->active;
    a.prefix = v->prefix;
    a.rel = v->rel;
    a.rel_off = v->rel_off;
    a.A = 0;
    return a;
}

extern "C" glint_status glint_server_step(glint_server *v, uint32_t *n_active, uint32_t *n_queued) {
    if (!v) return GLINT_ERR_INVALID_ARGUMENT;
    if (!v->ctx) return GLINT_ERR_STATE;
    glint_ctx *c = v->ctx;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    const uint32_t N = c->N;
    cudaError_t e;
    /* the kept blocks, as device descriptors */
    const uint32_t nb = (uint32_t)c->ctbs.size();
    if (v->blocks_cap < nb) {
        if (v->blocks) cudaFree(v->blocks);
        v->blocks = nullptr;
        v->blocks_cap = 0;
        if ((e = cudaMalloc((void **)&v->blocks, sizeof(StoreBlockDev) * nb)) != cudaSuccess)
            return server_fail(v, e, "blocks");
        v->blocks_cap = nb;
    }
    std::vector<StoreBlockDev> bd(nb);
    for (uint32_t i = 0; i < nb; ++i) {
        const StoreBlock &b = c->ctbs[i];
        bd[i] = StoreBlockDev{b.keys, b.key_bytes, b.ctfs, b.key_index, b.byte_index, b.sids, b.first, b.count,
                              b.okeys, b.end_time_min, b.C};
    }
    if (nb) cudaMemcpyAsync(v->blocks, bd.data(), sizeof(StoreBlockDev) * nb, cudaMemcpyHostToDevice, s);
    HopArgs a = server_args(v, nb);

    /* admission: queued queries into free slots */
    std::vector<uint32_t> admitted;
    std::vector<uint32_t> seeds;
    std::vector<unsigned long long> sprefix(1, 0);
    for (uint32_t k = 0; k < v->slots && !v->queue.empty(); ++k) {
        SlotState &st = v->state[k];
        if (st.busy) continue;
        PendingQuery q = std::move(v->queue.front());
        v->queue.pop_front();
        st = SlotState();
        st.busy = true;
        st.ticket = q.ticket;
        st.hops = q.hops;
        v->hparam[k] = SlotParam{q.t_start, q.t_end, (q.t_start == 0 && q.t_end == 0) ? 0u : 1u, 0u};
        admitted.push_back(k);
        seeds.insert(seeds.end(), q.seeds.begin(), q.seeds.end());
        sprefix.push_back(seeds.size());
    }
    if (!admitted.empty()) {
        if (v->seeds_cap < seeds.size()) {
            if (v->seeds) cudaFree(v->seeds);
            v->seeds = nullptr;
            v->seeds_cap = 0;
            if ((e = cudaMalloc((void **)&v->seeds, sizeof(uint32_t) * seeds.size())) != cudaSuccess)
                return server_fail(v, e, "seeds");
            v->seeds_cap = seeds.size();
        }
        for (uint32_t k : admitted) {
            cudaMemsetAsync(v->visited + (size_t)k * v->words, 0, sizeof(uint32_t) * v->words, s);
            cudaMemsetAsync(v->counts + k, 0, sizeof(uint32_t), s);
            cudaMemsetAsync(v->scanned + k, 0, sizeof(unsigned long long), s);
        }
        cudaMemcpyAsync(v->param, v->hparam.data(), sizeof(SlotParam) * v->slots, cudaMemcpyHostToDevice, s);
        if (!seeds.empty())
            cudaMemcpyAsync(v->seeds, seeds.data(), sizeof(uint32_t) * seeds.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->sprefix, sprefix.data(), sizeof(unsigned long long) * sprefix.size(),
                        cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->seed_slots, admitted.data(), sizeof(uint32_t) * admitted.size(), cudaMemcpyHostToDevice,
                        s);
        if (!seeds.empty())
            k_serve_seed<<<grid_for(seeds.size(), 256), 256, 0, s>>>(v->seeds, v->sprefix, v->seed_slots,
                                                                      (uint32_t)admitted.size(), a);
        std::vector<uint32_t> cnt(v->slots);
        cudaMemcpyAsync(cnt.data(), v->counts, sizeof(uint32_t) * v->slots, cudaMemcpyDeviceToHost, s);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return server_fail(v, e, "seed");
        for (uint32_t k : admitted) v->state[k].frontier = cnt[k];
    }

    /* one hop for every active slot, over the kept blocks that can hold a
     * key inside its window: a key of a block ends at most at end_time_max
     * and starts no earlier than start_min, and it counts when
     * start < t_end and t_start < end */
    std::vector<uint32_t> act, rel;
    std::vector<uint32_t> rel_off(1, 0);
    std::vector<unsigned long long> prefix(1, 0);
    for (uint32_t k = 0; k < v->slots; ++k) {
        const SlotState &st = v->state[k];
        if (!st.busy || st.hop >= st.hops) continue;
        act.push_back(k);
        const SlotParam &sp = v->hparam[k];
        uint32_t nrel = 0;
        for (uint32_t i = 0; i < nb; ++i) {
            const StoreBlock &b = c->ctbs[i];
            if (sp.window && b.spans_known && !(b.start_min < sp.t_end && sp.t_start < b.end_time_max)) continue;
            rel.push_back(i);
            ++nrel;
        }
        rel_off.push_back((uint32_t)rel.size());
        prefix.push_back(prefix.back() + (unsigned long long)st.frontier * nrel);
    }
    if (!act.empty()) {
        if (v->rel_cap < rel.size() + 1) {
            if (v->rel) cudaFree(v->rel);
            v->rel = nullptr;
            v->rel_cap = 0;
            if ((e = cudaMalloc((void **)&v->rel, sizeof(uint32_t) * (rel.size() + 1))) != cudaSuccess)
                return server_fail(v, e, "blocks of the windows");
            v->rel_cap = rel.size() + 1;
        }
        if (v->rel_off_cap < rel_off.size()) {
            if (v->rel_off) cudaFree(v->rel_off);
            v->rel_off = nullptr;
            v->rel_off_cap = 0;
            if ((e = cudaMalloc((void **)&v->rel_off, sizeof(uint32_t) * rel_off.size())) != cudaSuccess)
                return server_fail(v, e, "blocks of the windows");
            v->rel_off_cap = rel_off.size();
        }
        a.rel = v->rel;
        a.rel_off = v->rel_off;
        cudaMemcpyAsync(v->param, v->hparam.data(), sizeof(SlotParam) * v->slots, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->active, act.data(), sizeof(uint32_t) * act.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->prefix, prefix.data(), sizeof(unsigned long long) * prefix.size(), cudaMemcpyHostToDevice,
                        s);
        if (!rel.empty())
            cudaMemcpyAsync(v->rel, rel.data(), sizeof(uint32_t) * rel.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->rel_off, rel_off.data(), sizeof(uint32_t) * rel_off.size(), cudaMemcpyHostToDevice, s);
        for (uint32_t k : act) cudaMemsetAsync(v->counts + k, 0, sizeof(uint32_t), s);
        a.A = (uint32_t)act.size();
        const unsigned long long items = prefix.back();
        if (items) k_serve_hop<<<grid_for(items, 256, 152u * 16u), 256, 0, s>>>(a);
        std::vector<uint32_t> cnt(v->slots);
        std::vector<unsigned long long> scanned(v->slots);
        cudaMemcpyAsync(cnt.data(), v->counts, sizeof(uint32_t) * v->slots, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(scanned.data(), v->scanned, sizeof(unsigned long long) * v->slots, cudaMemcpyDeviceToHost, s);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return server_fail(v, e, "hop");
        /* the hop's new ids of every active slot, in (slot, id) order: one
         * sort and one copy for all of them */
        std::vector<unsigned long long> roff(act.size() + 1, 0);
        for (size_t i = 0; i < act.size(); ++i) roff[i + 1] = roff[i] + std::min(cnt[act[i]], N);
        const uint64_t total = roff.back();
        if (total) {
            if ((e = server_result_space(v, total, (uint32_t)act.size())) != cudaSuccess)
                return server_fail(v, e, "results");
            for (uint32_t k : act) v->hparam[k].cur ^= 1u; /* the lists the hop wrote */
            cudaMemcpyAsync(v->param, v->hparam.data(), sizeof(SlotParam) * v->slots, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(v->roff, roff.data(), sizeof(unsigned long long) * roff.size(), cudaMemcpyHostToDevice,
                            s);
            k_serve_collect<<<grid_for(total, 256), 256, 0, s>>>(v->lists, N, v->active, v->param, v->roff,
                                                                 (uint32_t)act.size(), v->rk, v->rv);
            for (uint32_t k : act) v->hparam[k].cur ^= 1u;
            const int bits = 32 + std::max(1, radix_bits_for(act.size() - 1));
            if ((e = radix_sort_u64(v->rk, v->rv, v->rk2, v->rv2, total, bits, v->rs_tmp, v->rscan, s)) !=
                cudaSuccess)
                return server_fail(v, e, "results sort");
            k_serve_ids<<<grid_for(total, 256), 256, 0, s>>>(v->rk, total, v->rids);
            v->buf.resize(total);
            cudaMemcpyAsync(v->buf.data(), v->rids, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost, s);
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return server_fail(v, e, "results");
        }
        for (size_t ai = 0; ai < act.size(); ++ai) {
            const uint32_t k = act[ai];
            SlotState &st = v->state[k];
            const uint32_t got = std::min(cnt[k], N);
            const uint32_t nl = v->hparam[k].cur ^ 1u;
            if (got) st.ids.insert(st.ids.end(), v->buf.begin() + roff[ai], v->buf.begin() + roff[ai + 1]);
            st.hop_end[st.hop] = st.ids.size();
            ++st.hop;
            st.frontier = got;
            v->hparam[k].cur = nl;
            if (st.hop >= st.hops || got == 0) {
                for (uint32_t h = st.hop; h < kMaxHops; ++h) st.hop_end[h] = st.ids.size();
                FinishedQuery f;
                f.ids = std::move(st.ids);
                std::memcpy(f.hop_end, st.hop_end, sizeof(f.hop_end));
                f.keys_scanned = scanned[k];
                v->done[st.ticket] = std::move(f);
                st = SlotState();
            }
        }
    }
    /* queries admitted with an empty frontier or zero kept blocks finish here */
    for (uint32_t k = 0; k < v->slots; ++k) {
        SlotState &st = v->state[k];
        if (st.busy && st.frontier == 0 && st.hop < st.hops) {
            for (uint32_t h = st.hop; h < kMaxHops; ++h) st.hop_end[h] = st.ids.size();
            FinishedQuery f;
            f.ids = std::move(st.ids);
            std::memcpy(f.hop_end, st.hop_end, sizeof(f.hop_end));
            f.keys_scanned = 0;
            v->done[st.ticket] = std::move(f);
            st = SlotState();
        }
    }
    if (n_active) {
        uint32_t n = 0;
        for (const SlotState &st : v->state) n += st.busy ? 1u : 0u;
        *n_active = n;
    }
    if (n_queued) *n_queued = (uint32_t)v->queue.size();
    return GLINT_OK;
}

extern "C" glint_status glint_server_poll(glint_server *v, uint64_t ticket, glint_query_result *r, int *done) {
    if (!v || !done) return GLINT_ERR_INVALID_ARGUMENT;
    auto it = v->done.find(ticket);
    if (it == v->done.end()) {
        *done = 0;
        return GLINT_OK;
    }
    *done = 1;
    if (r) {
        const FinishedQuery &f = it->second;
        r->n = f.ids.size();
        for (uint32_t h = 0; h < kMaxHops; ++h) r->hop_end[h] = f.hop_end[h];
        r->keys_scanned = f.keys_scanned;
        if (r->ids && r->cap) std::memcpy(r->ids, f.ids.data(), sizeof(uint32_t) * std::min<uint64_t>(r->cap, f.ids.size()));
    }
    v->done.erase(it);
    return GLINT_OK;
}

namespace glint {
void server_free_default(glint_ctx *c) {
    if (c->server) glint_server_destroy(c->server);
    c->server = nullptr;
}

void servers_detach(glint_ctx *c) {
    for (glint_server *v : c->servers) {
        server_release(v);
        v->visited = v->lists = v->counts = v->active = v->seed_slots = v->seeds = nullptr;
        v->param = nullptr;
        v->scanned = v->prefix = v->sprefix = nullptr;
        v->blocks = nullptr;
        v->rel = v->rel_off = nullptr;
        v->ctx = nullptr;
    }
    c->servers.clear();
}
} // namespace glint

/* a batch through the context's default server: all queries queued, steps
 * until every one has finished */
extern "C" glint_status glint_query_batch(glint_ctx *c, const glint_query *qs, uint32_t nq, glint_query_result *rs) {
    if (!c || (nq && (!qs || !rs))) return GLINT_ERR_INVALID_ARGUMENT;
    for (uint32_t q = 0; q < nq; ++q)
        if ((qs[q].n_seeds && !qs[q].seeds) || qs[q].hops == 0 || qs[q].hops > kMaxHops)
            return GLINT_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        c->last_error = std::string("query: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    if (!c->server) {
        const glint_status st = glint_server_create(c, 64, &c->server);
        if (st != GLINT_OK) return st;
    }
    glint_server *v = c->server;
    std::vector<uint64_t> tickets(nq);
    for (uint32_t q = 0; q < nq; ++q) glint_server_submit(v, &qs[q], &tickets[q]);
    uint32_t finished = 0;
    std::vector<char> got(nq, 0);
    while (finished < nq) {
        const glint_status st = glint_server_step(v, nullptr, nullptr);
        if (st != GLINT_OK) return st;
        for (uint32_t q = 0; q < nq; ++q) {
            if (got[q]) continue;
            int done = 0;
            glint_server_poll(v, tickets[q], &rs[q], &done);
            if (done) {
                got[q] = 1;
                ++finished;
            }
        }
    }
    return GLINT_OK;
}

extern "C" uint32_t glint_store_blocks(const glint_ctx *c) { return c ? (uint32_t)c->ctbs.size() : 0u; }
