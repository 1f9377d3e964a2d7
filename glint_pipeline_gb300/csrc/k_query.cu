/*
 * k_query.cu -- the active contact search (glint_active_search).
 *
 * Reference: with search_multi set, cuda_identify_meetings (cuda/geometry.cu:
 * 605-663) checks every bucket whose meeting is still active (end ==
 * cur_time) and has lasted cur_time - start >= min_meet_time + 1 against the
 * listed ids (search_multi_pid) and appends (pid, target, start, end, mbr)
 * records (search_info_unit, tracing/workbench.h:85-88) with an atomic
 * counter; tracing/process.cpp:465-475 prints them after the step.
 *
 * Device form, run after a step against the table it left: the listed ids
 * become a bitmap of N bits; pass 1 reads the stamp byte of every bucket and
 * the record only of buckets touched at the last step, and counts matching
 * sides per 8192-bucket tile; an exclusive scan gives each tile its offset;
 * pass 2 writes the records in bucket order.  The output order is therefore
 * deterministic.
 */
#include <algorithm>
#include <cstring>
#include <mutex>

#include "glint_internal.cuh"

namespace glint {

uint64_t identify_tiles(uint64_t B);

constexpr int kSearchThreads = 512;
constexpr int kSearchItems = 16;
constexpr uint32_t kSearchTile = kSearchThreads * kSearchItems; /* = the identify tile */

struct SearchArgs {
    const TRec *tab;
    const uint8_t *stamp;
    uint64_t B;
    uint8_t st;              /* stamp of entries touched at the last step */
    uint32_t cur_time;
    uint32_t min_plus1;
    const uint32_t *bits;
    uint32_t N;
};

__global__ void __launch_bounds__(256) k_search_set_bits(const uint32_t *__restrict__ pids, uint32_t n,
                                                         uint32_t *__restrict__ bits, uint32_t N) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = pids[i];
        if (p < N) atomicOr(&bits[p >> 5], 1u << (p & 31));
    }
}

__device__ inline bool listed(const SearchArgs &a, uint32_t p) {
    return p < a.N && ((a.bits[p >> 5] >> (p & 31)) & 1u);
}

/* matching sides of bucket `slot` touched at the last step: bit 0 the lower
 * id, bit 1 the higher id */
__device__ inline uint32_t search_sides(const SearchArgs &a, uint64_t slot, TRec &r) {
    r = a.tab[slot];
    if (r.w0 == kEmptyW0 || (r.w0 & kNewFlag)) return 0;
    if (a.cur_time - (uint32_t)r.w1 < a.min_plus1) return 0;
    return (listed(a, pair_a(r.w0)) ? 1u : 0u) | (listed(a, pair_b(r.w0)) ? 2u : 0u);
}

/* per thread: the sides mask of its 16 buckets, 2 bits each */
__device__ inline uint32_t search_thread_masks(const SearchArgs &a, uint64_t base) {
    uint32_t masks = 0;
    if (base >= a.B) return 0;
    const uint4 s4 = *reinterpret_cast<const uint4 *>(a.stamp + base); /* stamps padded to 16 */
    const uint32_t w[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
    for (int k = 0; k < kSearchItems; ++k) {
        if ((uint8_t)(w[k >> 2] >> (8 * (k & 3))) != a.st || base + k >= a.B) continue;
        TRec r;
        masks |= search_sides(a, base + k, r) << (2 * k);
    }
    return masks;
}

__global__ void __launch_bounds__(kSearchThreads) k_search_count(SearchArgs a, uint32_t *__restrict__ tile_cnt) {
    __shared__ uint32_t red[kSearchThreads / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kSearchTile + (uint64_t)threadIdx.x * kSearchItems;
    uint32_t v = (uint32_t)__popc(search_thread_masks(a, base));
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int i = 0; i < kSearchThreads / 32; ++i) t += red[i];
        tile_cnt[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kSearchThreads) k_search_emit(SearchArgs a, const uint32_t *__restrict__ tile_cnt,
                                                                const uint32_t *__restrict__ tile_off,
                                                                glint_search_info *__restrict__ out, uint64_t cap) {
    if (tile_cnt[blockIdx.x] == 0) return; /* uniform per block */
    __shared__ uint32_t ws[kSearchThreads / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kSearchTile + (uint64_t)threadIdx.x * kSearchItems;
    const uint32_t masks = search_thread_masks(a, base);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t v = (uint32_t)__popc(masks);
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < kSearchThreads / 32 ? ws[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kSearchThreads / 32) ws[lane] = s;
    }
    __syncthreads();
    if (!masks) return;
    uint64_t pos = (uint64_t)tile_off[blockIdx.x] + (wid ? ws[wid - 1] : 0u) + x - v;
    for (int k = 0; k < kSearchItems; ++k) {
        const uint32_t m = (masks >> (2 * k)) & 3u;
        if (!m) continue;
        const TRec r = a.tab[base + k];
        const uint32_t pa = pair_a(r.w0), pb = pair_b(r.w0);
        const uint4 mb = *reinterpret_cast<const uint4 *>(r.mbr);
        for (int side = 0; side < 2; ++side) {
            if (!(m & (1u << side))) continue;
            if (pos < cap) {
                glint_search_info o;
                o.pid = side ? pb : pa;
                o.target = side ? pa : pb;
                o.start = (uint32_t)r.w1;
                o.end = a.cur_time;
                o.mbr[0] = fdec(mb.x);
                o.mbr[1] = fdec(mb.y);
                o.mbr[2] = fdec(mb.z);
                o.mbr[3] = fdec(mb.w);
                out[pos] = o;
            }
            ++pos;
        }
    }
}

__global__ void k_search_total(const uint32_t *__restrict__ tile_off, uint64_t tiles, unsigned long long *n) {
    *n = tile_off[tiles];
}

SearchArgs search_args(const glint_ctx *c, const uint32_t *bits) {
    SearchArgs a;
    a.tab = c->d_tab;
    a.stamp = c->d_stamp;
    a.B = c->B;
    a.st = stamp_of(c->step_index);
    a.cur_time = c->last_time;
    a.min_plus1 = c->cfg.min_meet_time + 1;
    a.bits = bits;
    a.N = c->N;
    return a;
}

/* the search on the context's stream with caller-provided scratch:
 * bits[(N + 31) / 32] (cleared here), tile_cnt / tile_off [tiles + 1] and a
 * scan that maps tile_cnt -> tile_off */
template <class Scan>
cudaError_t launch_active_search(const glint_ctx *c, uint32_t *bits, uint32_t *tile_cnt, uint32_t *tile_off,
                                 Scan scan, const uint32_t *d_pids, uint32_t npids, glint_search_info *d_out,
                                 uint64_t cap, unsigned long long *d_n) {
    cudaStream_t s = c->stream;
    const uint64_t tiles = identify_tiles(c->B);
    cudaError_t e = cudaMemsetAsync(bits, 0, sizeof(uint32_t) * (((size_t)c->N + 31) / 32), s);
    if (e != cudaSuccess) return e;
    if (npids) k_search_set_bits<<<grid_for(npids, 256, 152u * 4u), 256, 0, s>>>(d_pids, npids, bits, c->N);
    const SearchArgs a = search_args(c, bits);
    k_search_count<<<(unsigned)tiles, kSearchThreads, 0, s>>>(a, tile_cnt);
    if ((e = scan(tile_cnt, tile_off, tiles, s)) != cudaSuccess) return e;
    k_search_emit<<<(unsigned)tiles, kSearchThreads, 0, s>>>(a, tile_cnt, tile_off, d_out, cap);
    k_search_total<<<1, 1, 0, s>>>(tile_off, tiles, d_n);
    return cudaGetLastError();
}

} // namespace glint

using namespace glint;

namespace {

template <class T>
cudaError_t grow(T **p, uint64_t &have, uint64_t need) {
    if (need <= have && *p) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    have = 0;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (need ? need : 1));
    if (e == cudaSuccess) have = need;
    return e;
}

} // namespace

extern "C" glint_status glint_active_search(glint_ctx *c, const uint32_t *pids, uint32_t npids, glint_search_info *out,
                                            uint64_t cap, uint64_t *n) {
    if (!c || (npids && !pids) || (cap && !out)) return GLINT_ERR_INVALID_ARGUMENT;
    if (c->step_index == 0) {
        c->last_error = "active search before the first step";
        return GLINT_ERR_STATE;
    }
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    const uint64_t words = ((uint64_t)c->N + 31) / 32;
    if (e == cudaSuccess) e = grow(&c->d_qbits, c->qbits_cap, words);
    if (e == cudaSuccess) e = grow(&c->d_qpids, c->qpids_cap, std::max<uint64_t>(npids, 1));
    if (e == cudaSuccess) e = grow(&c->d_qout, c->qout_cap, std::max<uint64_t>(cap, 1));
    if (e == cudaSuccess && !c->d_qn) e = cudaMalloc((void **)&c->d_qn, sizeof(unsigned long long));
    if (e == cudaSuccess && npids)
        e = cudaMemcpyAsync(c->d_qpids, pids, sizeof(uint32_t) * npids, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        void *tmp = c->d_scan_tmp;
        auto scan = [tmp](const uint32_t *in, uint32_t *o, uint64_t m, cudaStream_t s) {
            return scan_u32(in, o, m, tmp, s);
        };
        e = launch_active_search(c, c->d_qbits, c->d_tile_cnt, c->d_tile_off, scan, c->d_qpids, npids, c->d_qout, cap,
                                 c->d_qn);
    }
    unsigned long long found = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&found, c->d_qn, sizeof(found), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && found && cap)
        e = cudaMemcpy(out, c->d_qout, sizeof(glint_search_info) * std::min<uint64_t>(found, cap),
                       cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        c->last_error = std::string("active search: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    if (n) *n = found;
    return GLINT_OK;
}

/* ---- allocation-free variant --------------------------------------------
 * glint_active_search_noalloc takes device arrays and keeps its scratch in
 * one fixed-size device array of this library: the id bitmap (objects up to
 * kNaMaxObjects) and the per-tile counts and offsets (buckets up to
 * kNaMaxTiles * 8192).  Its address is looked up once per device while a
 * context is created on it; the call itself allocates nothing. */
namespace glint {

constexpr uint32_t kNaMaxObjects = 1u << 24;                 /* 16.7M objects: 2 MB of bits */
constexpr uint32_t kNaMaxTiles = 1u << 17;                   /* 2^30 buckets: 2 x 512 KB */
constexpr size_t kNaBitsWords = kNaMaxObjects / 32;
constexpr size_t kNaTileWords = (size_t)kNaMaxTiles + 64;    /* tiles + 1, padded to 256 B */
constexpr size_t kNaWords = kNaBitsWords + 2 * kNaTileWords;
constexpr int kNaMaxDevices = 64;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaWords];

std::mutex g_na_mutex;
uint32_t *g_na_ptr[kNaMaxDevices];
cudaError_t g_na_status[kNaMaxDevices];
bool g_na_done[kNaMaxDevices];

/* exclusive scan of n (<= kNaMaxTiles + 1) values by one block, no scratch */
__global__ void __launch_bounds__(1024) k_scan_one_block(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                         uint64_t n) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < n; base += blockDim.x) {
        const uint64_t i = base + threadIdx.x;
        const uint32_t v = i < n ? in[i] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = ws[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            ws[lane] = s;
        }
        __syncthreads();
        const uint32_t excl = carry + (wid ? ws[wid - 1] : 0u) + x - v;
        if (i < n) out[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += ws[31];
        __syncthreads();
    }
}

/* looks up the scratch address on the current device, once per device */
cudaError_t noalloc_setup(int device) {
    if (device < 0 || device >= kNaMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_done[device]) {
        void *p = nullptr;
        g_na_status[device] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        g_na_ptr[device] = g_na_status[device] == cudaSuccess ? static_cast<uint32_t *>(p) : nullptr;
        g_na_done[device] = true;
    }
    return g_na_status[device];
}

} // namespace glint

extern "C" glint_status glint_active_search_noalloc(glint_ctx *c, const uint32_t *d_pids, uint32_t npids,
                                                    glint_search_info *d_out, uint64_t cap, uint64_t *d_n) {
    if (!c || (npids && !d_pids) || (cap && !d_out) || !d_n) return GLINT_ERR_INVALID_ARGUMENT;
    if (c->step_index == 0) {
        c->last_error = "active search before the first step";
        return GLINT_ERR_STATE;
    }
    if (c->N > kNaMaxObjects || identify_tiles(c->B) > kNaMaxTiles) {
        c->last_error = "glint_active_search_noalloc: context larger than its fixed scratch (objects <= 2^24, "
                        "buckets <= 2^30); use glint_active_search";
        return GLINT_ERR_UNSUPPORTED;
    }
    uint32_t *base = nullptr;
    cudaError_t st = cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (c->device >= 0 && c->device < kNaMaxDevices && g_na_done[c->device]) {
            st = g_na_status[c->device];
            base = g_na_ptr[c->device];
        }
    }
    if (st != cudaSuccess || !base) {
        c->last_error = std::string("glint_active_search_noalloc: scratch lookup failed: ") + cudaGetErrorString(st);
        return GLINT_ERR_CUDA;
    }
    cudaSetDevice(c->device);
    uint32_t *bits = base;
    uint32_t *tile_cnt = base + kNaBitsWords;
    uint32_t *tile_off = tile_cnt + kNaTileWords;
    auto scan = [](const uint32_t *in, uint32_t *o, uint64_t m, cudaStream_t s) {
        k_scan_one_block<<<1, 1024, 0, s>>>(in, o, m + 1);
        return cudaGetLastError();
    };
    static_assert(sizeof(uint64_t) == sizeof(unsigned long long), "u64");
    const cudaError_t e = launch_active_search(c, bits, tile_cnt, tile_off, scan, d_pids, npids, d_out, cap,
                                               reinterpret_cast<unsigned long long *>(d_n));
    if (e != cudaSuccess) {
        c->last_error = std::string("glint_active_search_noalloc: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    return GLINT_OK;
}

/* ---- contact-trace queries over the flushed store -------------------------
 * Breadth-first expansion for a batch of queries at once.  Per query slot: a
 * visited bitmap over objects and two object lists (this hop's frontier and
 * the next).  One launch per hop covers every (query, frontier object,
 * block) triple: the object's sid in the block gives its CTF (or the
 * oversize buffer), first/count its keys, and each key is decoded as the
 * reference's CTF::parse_key does (tracing/step_merge.cpp:335-345). */
namespace glint {

constexpr uint32_t kQuerySlots = 64;
constexpr uint32_t kMaxHops = 8;

struct HopArgs {
    const StoreBlockDev *blocks;
    uint32_t nblocks;
    uint32_t N;
    uint64_t words;                      /* bitmap words per slot */
    uint32_t *visited;
    uint32_t *lists;                     /* [slot][2][N] */
    uint32_t cur;                        /* which list is the frontier */
    const unsigned long long *prefix;    /* [Q + 1] frontier sizes, prefix sums */
    const uint32_t *qparam;              /* [Q][4] t_start, t_end, window */
    uint32_t *counts;                    /* [Q] next-list sizes */
    uint32_t Q;
    unsigned long long *scanned;
};

__device__ inline void visit(const HopArgs &a, uint32_t q, uint32_t target) {
    if (target >= a.N) return;
    uint32_t *vis = a.visited + (size_t)q * a.words;
    const uint32_t bit = 1u << (target & 31);
    const uint32_t old = atomicOr(&vis[target >> 5], bit);
    if (old & bit) return;
    const uint32_t idx = atomicAdd(&a.counts[q], 1u);
    if (idx < a.N) a.lists[((size_t)q * 2 + (a.cur ^ 1)) * a.N + idx] = target;
}

__global__ void __launch_bounds__(256) k_q_hop(HopArgs a) {
    const unsigned long long total = a.prefix[a.Q] * a.nblocks;
    unsigned long long scanned = 0;
    for (unsigned long long it = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; it < total;
         it += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long f = it / a.nblocks;
        const uint32_t b = (uint32_t)(it - f * a.nblocks);
        uint32_t lo = 0, hi = a.Q; /* the query: prefix[q] <= f < prefix[q + 1] */
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (a.prefix[mid] <= f) lo = mid;
            else hi = mid;
        }
        const uint32_t q = lo;
        const uint32_t obj = a.lists[((size_t)q * 2 + a.cur) * a.N + (f - a.prefix[q])];
        const StoreBlockDev blk = a.blocks[b];
        const uint32_t sid = blk.sids[obj];
        if (sid == 0) continue;
        const uint32_t n = blk.count[obj], first = blk.first[obj];
        const uint32_t t0 = a.qparam[4 * q], t1 = a.qparam[4 * q + 1], window = a.qparam[4 * q + 2];
        scanned += n;
        if (sid == 1) {
            for (uint32_t j = 0; j < n; ++j) {
                const ulonglong2 k = blk.okeys[first + j];
                const uint32_t end = (uint32_t)k.x + blk.end_time_min, duration = (uint32_t)(k.x >> 32);
                const uint32_t start = end - duration;
                if (window && !(start < t1 && t0 < end)) continue;
                visit(a, q, (uint32_t)k.y & ((1u << 26) - 1));
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
            unsigned __int128 v = 0;
            for (uint32_t t = 0; t < kb; ++t) v |= (unsigned __int128)p[t] << (8 * t);
            v >>= m.mbr_bit;
            const uint32_t end = (uint32_t)(v & ((1ull << m.end_bit) - 1)) + blk.end_time_min;
            v >>= m.end_bit;
            const uint32_t duration = (uint32_t)(v & ((1ull << m.duration_bit) - 1));
            v >>= m.duration_bit;
            const uint32_t target = (uint32_t)(v & ((1ull << m.id_bit) - 1));
            const uint32_t start = end - duration;
            if (window && !(start < t1 && t0 < end)) continue;
            visit(a, q, target);
        }
    }
    for (int o = 16; o > 0; o >>= 1) scanned += __shfl_down_sync(0xffffffffu, scanned, o);
    if ((threadIdx.x & 31) == 0 && scanned) atomicAdd(a.scanned, scanned);
}

/* the seeds of every query: visited and listed as the first frontier */
__global__ void k_q_seed(const uint32_t *__restrict__ seeds, const unsigned long long *__restrict__ sprefix, uint32_t Q,
                         HopArgs a) {
    const unsigned long long total = sprefix[Q];
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = Q;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (sprefix[mid] <= i) lo = mid;
            else hi = mid;
        }
        const uint32_t p = seeds[i];
        if (p >= a.N) continue;
        uint32_t *vis = a.visited + (size_t)lo * a.words;
        const uint32_t bit = 1u << (p & 31);
        if (atomicOr(&vis[p >> 5], bit) & bit) continue;
        const uint32_t idx = atomicAdd(&a.counts[lo], 1u);
        a.lists[((size_t)lo * 2 + a.cur) * a.N + idx] = p;
    }
}

void query_pool_free(glint_ctx *c) {
    QueryPool &p = c->qpool;
    void *ps[] = {p.visited, p.lists, p.counts, p.seeds, p.prefix, p.qparam, p.blocks};
    for (void *x : ps)
        if (x) cudaFree(x);
    p = QueryPool();
}

static cudaError_t query_pool_ensure(glint_ctx *c, uint32_t slots, uint64_t nseeds, uint32_t nblocks) {
    QueryPool &p = c->qpool;
    const uint64_t words = ((uint64_t)c->N + 31) / 32;
    cudaError_t e = cudaSuccess;
    if (p.slots < slots) {
        void *ps[] = {p.visited, p.lists, p.counts, p.prefix, p.qparam};
        for (void *x : ps)
            if (x) cudaFree(x);
        p.visited = p.lists = p.counts = p.qparam = nullptr;
        p.prefix = nullptr;
        p.slots = 0;
        if ((e = cudaMalloc((void **)&p.visited, sizeof(uint32_t) * words * slots)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void **)&p.lists, sizeof(uint32_t) * 2 * (size_t)c->N * slots)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void **)&p.counts, sizeof(uint32_t) * slots)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void **)&p.prefix, sizeof(unsigned long long) * (2 * (slots + 1) + 1))) != cudaSuccess)
            return e;
        if ((e = cudaMalloc((void **)&p.qparam, sizeof(uint32_t) * 4 * slots)) != cudaSuccess) return e;
        p.slots = slots;
    }
    if (p.seeds_cap < nseeds) {
        if (p.seeds) cudaFree(p.seeds);
        p.seeds = nullptr;
        p.seeds_cap = 0;
        if ((e = cudaMalloc((void **)&p.seeds, sizeof(uint32_t) * (nseeds ? nseeds : 1))) != cudaSuccess) return e;
        p.seeds_cap = nseeds;
    }
    if (p.blocks_cap < nblocks) {
        if (p.blocks) cudaFree(p.blocks);
        p.blocks = nullptr;
        p.blocks_cap = 0;
        if ((e = cudaMalloc((void **)&p.blocks, sizeof(StoreBlockDev) * (nblocks ? nblocks : 1))) != cudaSuccess)
            return e;
        p.blocks_cap = nblocks;
    }
    return e;
}

/* one batch of at most kQuerySlots queries */
static glint_status query_chunk(glint_ctx *c, const glint_query *qs, uint32_t Q, glint_query_result *rs) {
    cudaStream_t s = c->stream;
    const uint32_t nb = (uint32_t)c->ctbs.size();
    uint64_t nseeds = 0;
    uint32_t max_hops = 0;
    for (uint32_t q = 0; q < Q; ++q) {
        nseeds += qs[q].n_seeds;
        max_hops = std::max(max_hops, std::min(qs[q].hops, kMaxHops));
    }
    cudaError_t e = query_pool_ensure(c, Q, nseeds, nb);
    if (e != cudaSuccess) {
        c->last_error = std::string("query scratch: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    QueryPool &p = c->qpool;
    std::vector<StoreBlockDev> bd(nb);
    for (uint32_t i = 0; i < nb; ++i) {
        const StoreBlock &b = c->ctbs[i];
        bd[i] = StoreBlockDev{b.keys, b.ctfs, b.key_index, b.byte_index, b.sids, b.first, b.count, b.okeys,
                              b.end_time_min, c->cfg.CTF_count};
    }
    std::vector<uint32_t> seeds(nseeds ? nseeds : 1), qparam(4 * Q);
    std::vector<unsigned long long> sprefix(Q + 1), prefix(Q + 1);
    uint64_t at = 0;
    for (uint32_t q = 0; q < Q; ++q) {
        sprefix[q] = at;
        if (qs[q].n_seeds) std::memcpy(seeds.data() + at, qs[q].seeds, sizeof(uint32_t) * qs[q].n_seeds);
        at += qs[q].n_seeds;
        qparam[4 * q] = qs[q].t_start;
        qparam[4 * q + 1] = qs[q].t_end;
        qparam[4 * q + 2] = (qs[q].t_start == 0 && qs[q].t_end == 0) ? 0u : 1u;
        rs[q].n = 0;
        rs[q].keys_scanned = 0;
        for (uint32_t h = 0; h < kMaxHops; ++h) rs[q].hop_end[h] = 0;
    }
    sprefix[Q] = at;
    const uint64_t words = ((uint64_t)c->N + 31) / 32;
    unsigned long long *d_sprefix = p.prefix + (Q + 1);
    unsigned long long *d_scanned = p.prefix + 2 * (Q + 1);
    cudaMemsetAsync(d_scanned, 0, sizeof(unsigned long long), s);
    cudaMemsetAsync(p.visited, 0, sizeof(uint32_t) * words * Q, s);
    cudaMemsetAsync(p.counts, 0, sizeof(uint32_t) * Q, s);
    if (nb) cudaMemcpyAsync(p.blocks, bd.data(), sizeof(StoreBlockDev) * nb, cudaMemcpyHostToDevice, s);
    if (nseeds) cudaMemcpyAsync(p.seeds, seeds.data(), sizeof(uint32_t) * nseeds, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_sprefix, sprefix.data(), sizeof(unsigned long long) * (Q + 1), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p.qparam, qparam.data(), sizeof(uint32_t) * 4 * Q, cudaMemcpyHostToDevice, s);
    HopArgs a;
    a.blocks = p.blocks;
    a.nblocks = nb;
    a.N = c->N;
    a.words = words;
    a.visited = p.visited;
    a.lists = p.lists;
    a.cur = 0;
    a.prefix = p.prefix;
    a.qparam = p.qparam;
    a.counts = p.counts;
    a.Q = Q;
    a.scanned = d_scanned;
    if (nseeds) k_q_seed<<<grid_for(nseeds, 256), 256, 0, s>>>(p.seeds, d_sprefix, Q, a);
    std::vector<uint32_t> cnt(Q);
    cudaMemcpyAsync(cnt.data(), p.counts, sizeof(uint32_t) * Q, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
        c->last_error = std::string("query seeds: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    std::vector<uint32_t> buf;
    for (uint32_t h = 0; h < max_hops; ++h) {
        /* frontier sizes; finished queries expand nothing */
        unsigned long long acc = 0;
        for (uint32_t q = 0; q < Q; ++q) {
            prefix[q] = acc;
            acc += (h < qs[q].hops) ? cnt[q] : 0u;
        }
        prefix[Q] = acc;
        cudaMemcpyAsync(p.prefix, prefix.data(), sizeof(unsigned long long) * (Q + 1), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(p.counts, 0, sizeof(uint32_t) * Q, s);
        a.cur = h & 1;
        if (acc && nb) k_q_hop<<<grid_for(acc * nb, 256, 152u * 16u), 256, 0, s>>>(a);
        cudaMemcpyAsync(cnt.data(), p.counts, sizeof(uint32_t) * Q, cudaMemcpyDeviceToHost, s);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        for (uint32_t q = 0; q < Q; ++q) {
            if (h >= qs[q].hops) {
                cnt[q] = 0;
                continue;
            }
            const uint32_t k = std::min(cnt[q], c->N);
            glint_query_result &r = rs[q];
            if (k) {
                buf.resize(k);
                e = cudaMemcpy(buf.data(), p.lists + ((size_t)q * 2 + (a.cur ^ 1)) * c->N, sizeof(uint32_t) * k,
                               cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) break;
                std::sort(buf.begin(), buf.end());
                for (uint32_t i = 0; i < k; ++i)
                    if (r.ids && r.n + i < r.cap) r.ids[r.n + i] = buf[i];
            }
            r.n += k;
            r.hop_end[h] = r.n;
        }
        if (e != cudaSuccess) break;
    }
    unsigned long long scanned = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&scanned, d_scanned, sizeof(scanned), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        c->last_error = std::string("query: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    for (uint32_t q = 0; q < Q; ++q) {
        rs[q].keys_scanned = q == 0 ? scanned : 0; /* per batch, reported on its first query */
        for (uint32_t h = std::min(qs[q].hops, kMaxHops); h < kMaxHops; ++h) rs[q].hop_end[h] = rs[q].n;
    }
    return GLINT_OK;
}

} // namespace glint

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
    for (uint32_t b = 0; b < nq; b += kQuerySlots) {
        const glint_status st = query_chunk(c, qs + b, std::min(kQuerySlots, nq - b), rs + b);
        if (st != GLINT_OK) return st;
    }
    return GLINT_OK;
}

extern "C" uint32_t glint_store_blocks(const glint_ctx *c) { return c ? (uint32_t)c->ctbs.size() : 0u; }
