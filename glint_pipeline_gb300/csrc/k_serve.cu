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
    const uint32_t *front;                 /* [A] their frontier sizes */
    const unsigned long long *prefix;      /* [A + 1] their items (frontier x blocks), prefix sums */
    const uint32_t *rel;                   /* each active slot's blocks, concatenated */
    const uint32_t *rel_off;               /* [A + 1] where each active slot's blocks start in rel */
    uint32_t A;
};

/* the reached-set word of target for slot s (all ones past N) */
__device__ inline uint32_t visited_word(const HopArgs &a, uint32_t s, uint32_t target) {
    return target < a.N ? __ldcg(&a.visited[(size_t)s * a.words + (target >> 5)]) : ~0u;
}

/* marks target reached for slot s and appends it to the slot's next list
 * when it is new, given its reached-set word `seen` (visited_word); the
 * lanes that call together and append to the same slot take their places
 * with one atomic (a slot's counter is one address that every new object of
 * a large frontier would otherwise hit) */
__device__ inline void visit_seen(const HopArgs &a, uint32_t s, uint32_t next_list, uint32_t target, uint32_t seen) {
    const unsigned calling = __activemask();
    bool fresh = false;
    if (target < a.N) {
        /* a query's bits only go from 0 to 1, so a set bit read from L2 is
         * final and saves the atomic; a clear one is settled by the atomic */
        const uint32_t bit = 1u << (target & 31);
        if (!(seen & bit)) fresh = !(atomicOr(&a.visited[(size_t)s * a.words + (target >> 5)], bit) & bit);
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

/* one item's keys as the hop reads them: where they start, how many, and
 * how a key decodes (kind 1: the oversize buffer's 16-byte keys; kind 2: a
 * CTF's packed keys, whose end, duration and target fields lie in the 64
 * bits from byte off of the key when fast is set) */
struct HopItem {
    const uint8_t *base;
    const uint8_t *end;      /* the end of the block's packed keys */
    uint32_t n, s, nl, kind;
    uint32_t kb, off, fast, mbr_bit;
    uint32_t end_bit, dur_bit, end_mask, dur_mask;
    uint32_t id_mask, etm, window, t_start;
    uint32_t t_end, pad0, pad1, pad2;
};

constexpr int kHopThreads = 256;
constexpr int kHopKeys = 4; /* keys per lane per round */

/* the 64 bits at p, which need not be aligned; whole words while they stay
 * inside the buffer ending at `end` (whose start is 8-aligned) */
__device__ inline unsigned long long load_u64(const uint8_t *p, const uint8_t *end) {
    const uintptr_t a = (uintptr_t)p;
    const uint64_t *w = (const uint64_t *)(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7) * 8;
    if ((const uint8_t *)(w + 2) <= end) {
        const uint64_t lo = w[0];
        return sh ? (lo >> sh) | (w[1] << (64 - sh)) : lo;
    }
    unsigned long long v = 0;
    for (uint32_t i = 0; i < 8 && p + i < end; ++i) v |= (unsigned long long)p[i] << (8 * i);
    return v;
}

/* Each warp takes 32 consecutive items, one per lane, and looks up the
 * object's sid, first key and key count in the item's block.  An object has
 * anywhere from none to hundreds of keys in a block, so the warp then walks
 * the keys of all 32 items together, 32 at a time: lane l takes the warp's
 * key k0 + l, finds its item by a binary search over the items' key counts'
 * prefix sums, and reads that item's decoding from shared memory.  Every lane
 * has a key on every round but the last, and the warp's loop count is its
 * total keys / 32 instead of its largest item's key count.  A lane decodes
 * kHopKeys keys before it reads their bitmap words, so that their loads
 * overlap. */
__global__ void __launch_bounds__(kHopThreads) k_serve_hop(HopArgs a) {
    __shared__ HopItem items[kHopThreads];
    __shared__ uint32_t koff[kHopThreads];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    HopItem *wi = items + wib * 32;
    uint32_t *wo = koff + wib * 32;
    const unsigned long long total = a.prefix[a.A];
    const unsigned long long warps = (unsigned long long)gridDim.x * (kHopThreads / 32);
    for (unsigned long long w = blockIdx.x * (unsigned long long)(kHopThreads / 32) + wib; w * 32 < total;
         w += warps) {
        const unsigned long long it = w * 32 + lane;
        HopItem h;
        h.n = 0;
        h.kind = 0;
        h.s = 0;
        if (it < total) {
            uint32_t lo = 0, hi = a.A; /* prefix[lo] <= it < prefix[lo + 1] */
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) / 2;
                if (a.prefix[mid] <= it) lo = mid;
                else hi = mid;
            }
            /* block-major within a slot: consecutive items take consecutive
             * frontier objects (ascending ids) of one block, whose sids,
             * key ranges and keys then lie close together */
            const uint32_t fr = a.front[lo];
            const unsigned long long local = it - a.prefix[lo];
            uint32_t bi, f;
            if (local < (1ull << 32)) {
                bi = (uint32_t)local / fr;
                f = (uint32_t)local - bi * fr;
            } else {
                bi = (uint32_t)(local / fr);
                f = (uint32_t)(local - (unsigned long long)bi * fr);
            }
            const uint32_t b = a.rel[a.rel_off[lo] + bi];
            const uint32_t s = a.active[lo];
            const SlotParam sp = a.param[s];
            const uint32_t obj = a.lists[((size_t)s * 2 + sp.cur) * a.N + f];
            const StoreBlockDev &blk = a.blocks[b];
            const uint32_t sid = blk.sids[obj];
            h.s = s;
            h.nl = sp.cur ^ 1u;
            h.window = sp.window;
            h.t_start = sp.t_start;
            h.t_end = sp.t_end;
            h.etm = blk.end_time_min;
            if (sid == 1) {
                h.n = blk.count[obj];
                h.kind = 1;
                h.base = reinterpret_cast<const uint8_t *>(blk.okeys + blk.first[obj]);
            } else if (sid >= 2 && sid - 2 < blk.C) {
                const uint32_t c = sid - 2;
                const glint_ctf_meta &m = blk.ctfs[c];
                const uint32_t kb = m.key_bit / 8, mb = m.mbr_bit, eb = m.end_bit, db = m.duration_bit,
                               ib = m.id_bit;
                h.n = blk.count[obj];
                h.kind = 2;
                h.kb = kb;
                h.mbr_bit = mb;
                h.off = mb / 8;
                h.fast = (mb & 7) + eb + db + ib <= 64;
                h.end_bit = eb;
                h.dur_bit = db;
                h.end_mask = eb >= 32 ? 0xffffffffu : (1u << eb) - 1u;
                h.dur_mask = db >= 32 ? 0xffffffffu : (1u << db) - 1u;
                h.id_mask = ib >= 32 ? 0xffffffffu : (1u << ib) - 1u;
                h.end = blk.keys + blk.key_bytes;
                h.base = blk.keys + blk.byte_index[c] + (unsigned long long)(blk.first[obj] - blk.key_index[c]) * kb;
            }
        }
        /* keys read, per slot: the lanes of one slot add with one reduction */
        const unsigned withkeys = __ballot_sync(0xffffffffu, h.n != 0);
        if (h.n) {
            const unsigned peers = __match_any_sync(withkeys, h.s);
            const uint32_t grp = __reduce_add_sync(peers, h.n);
            if (lane == __ffs(peers) - 1) atomicAdd(&a.scanned[h.s], (unsigned long long)grp);
        }
        /* exclusive prefix of the key counts over the warp */
        uint32_t incl = h.n;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const uint32_t T = __shfl_sync(0xffffffffu, incl, 31);
        wi[lane] = h;
        wo[lane] = incl - h.n;
        __syncwarp();
        /* kHopKeys keys per lane in flight: their loads, then their bitmap
         * words, then the (rare) atomics and appends */
        for (uint32_t k0 = 0; k0 < T; k0 += 32 * kHopKeys) {
            uint32_t tg[kHopKeys], sl[kHopKeys], nx[kHopKeys], seen[kHopKeys];
#pragma unroll
            for (int u = 0; u < kHopKeys; ++u) {
                const uint32_t k = k0 + u * 32 + lane;
                tg[u] = 0xffffffffu;
                sl[u] = 0;
                nx[u] = 0;
                if (k < T) {
                    /* the last item whose first key is at or before k: it has
                     * keys, since an item without keys shares its offset with
                     * the item after it, and k < T rules out the last lane */
                    uint32_t lo = 0;
#pragma unroll
                    for (uint32_t step = 16; step; step >>= 1)
                        if (lo + step < 32 && wo[lo + step] <= k) lo += step;
                    const HopItem &x = wi[lo];
                    const uint32_t j = k - wo[lo];
                    sl[u] = x.s;
                    nx[u] = x.nl;
                    uint32_t end, duration, t;
                    if (x.kind == 2 && x.fast) {
                        /* end, duration and target from one 64-bit window */
                        unsigned long long v = load_u64(x.base + (size_t)j * x.kb + x.off, x.end);
                        v >>= x.mbr_bit & 7;
                        end = ((uint32_t)v & x.end_mask) + x.etm;
                        v >>= x.end_bit;
                        duration = (uint32_t)v & x.dur_mask;
                        v >>= x.dur_bit;
                        t = (uint32_t)v & x.id_mask;
                    } else if (x.kind == 2) {
                        unsigned __int128 v = load_key(x.base + (size_t)j * x.kb, x.kb, x.end);
                        v >>= x.mbr_bit;
                        end = (uint32_t)(v & ((1ull << x.end_bit) - 1)) + x.etm;
                        v >>= x.end_bit;
                        duration = (uint32_t)(v & ((1ull << x.dur_bit) - 1));
                        v >>= x.dur_bit;
                        t = (uint32_t)v & x.id_mask;
                    } else {
                        const ulonglong2 kk = reinterpret_cast<const ulonglong2 *>(x.base)[j];
                        end = (uint32_t)kk.x + x.etm;
                        duration = (uint32_t)(kk.x >> 32);
                        t = (uint32_t)kk.y & ((1u << 26) - 1);
                    }
                    const uint32_t start = end - duration;
                    if (!x.window || (start < x.t_end && x.t_start < end)) tg[u] = t;
                }
            }
#pragma unroll
            for (int u = 0; u < kHopKeys; ++u) seen[u] = visited_word(a, sl[u], tg[u]);
#pragma unroll
            for (int u = 0; u < kHopKeys; ++u) visit_seen(a, sl[u], nx[u], tg[u], seen[u]);
        }
        __syncwarp();
    }
}

/* ---- pull hops -----------------------------------------------------------
 * When a slot's frontier is at least as large as the set of objects it has
 * not reached, the hop runs from the other side: every unreached object u
 * reads its own keys in the window's blocks and is reached when one of its
 * targets was reached before this hop.  A meeting's two keys (a -> b and
 * b -> a, cuda/geometry.cu:714-734) lie in the same block with the same
 * times, so u has a key to a reached object v exactly when v has one to u;
 * and v was reached at the previous hop, since a v reached earlier would have
 * reached u already.  The reached set is read as it stood before the hop
 * (its bits are set after it, k_serve_mark), so the hop's result is the one
 * the frontier's own walk gives, and u stops at its first such key. */

/* the unreached objects of pull slot blockIdx.y into its frontier list,
 * ascending within each warp's 1024 ids */
__global__ void __launch_bounds__(256) k_serve_unvisited(HopArgs b, unsigned int *ucount) {
    const uint32_t s = b.active[blockIdx.y];
    const uint32_t *vis = b.visited + (size_t)s * b.words;
    uint32_t *out = b.lists + ((size_t)s * 2 + b.param[s].cur) * b.N;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (b.N + 31) / 32;
    for (uint32_t w0 = blockIdx.x * blockDim.x; w0 < nw; w0 += gridDim.x * blockDim.x) {
        const uint32_t w = w0 + threadIdx.x;
        uint32_t inv = 0;
        if (w < nw) {
            inv = ~vis[w];
            if (w == nw - 1 && (b.N & 31)) inv &= (1u << (b.N & 31)) - 1u;
        }
        const uint32_t k = __popc(inv);
        uint32_t incl = k;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t base = 0;
        if (lane == 31 && incl) base = atomicAdd(&ucount[s], incl);
        base = __shfl_sync(0xffffffffu, base, 31);
        uint32_t at = base + incl - k;
        while (inv) {
            const int bit = __ffs(inv) - 1;
            inv &= inv - 1u;
            if (at < b.N) out[at] = w * 32 + (uint32_t)bit;
            ++at;
        }
    }
}

/* one warp per unreached object: its keys in the slot's blocks, 32 blocks
 * at a time, until one reaches an object reached before this hop */
__global__ void __launch_bounds__(256) k_serve_pull(HopArgs b) {
    const int lane = threadIdx.x & 31;
    const unsigned long long total = b.prefix[b.A];
    const unsigned long long nwarps = (unsigned long long)gridDim.x * (blockDim.x / 32);
    for (unsigned long long w = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) / 32; w < total;
         w += nwarps) {
        uint32_t lo = 0, hi = b.A; /* prefix[lo] <= w < prefix[lo + 1] */
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (b.prefix[mid] <= w) lo = mid;
            else hi = mid;
        }
        const uint32_t s = b.active[lo];
        const SlotParam sp = b.param[s];
        const uint32_t u = b.lists[((size_t)s * 2 + sp.cur) * b.N + (w - b.prefix[lo])];
        const uint32_t *vis = b.visited + (size_t)s * b.words;
        const uint32_t r0 = b.rel_off[lo], nrel = b.rel_off[lo + 1] - r0;
        bool found = false;
        unsigned long long keys = 0;
        for (uint32_t r = 0; r < nrel && !found; r += 32) {
            bool hit = false;
            if (r + lane < nrel) {
                const StoreBlockDev &blk = b.blocks[b.rel[r0 + r + lane]];
                const uint32_t sid = blk.sids[u];
                uint32_t n = 0;
                if (sid == 1) {
                    n = blk.count[u];
                    const ulonglong2 *k = blk.okeys + blk.first[u];
                    for (uint32_t j = 0; j < n && !hit; ++j) {
                        const ulonglong2 kk = k[j];
                        const uint32_t end = (uint32_t)kk.x + blk.end_time_min, dur = (uint32_t)(kk.x >> 32);
                        const uint32_t t = (uint32_t)kk.y & ((1u << 26) - 1);
                        ++keys;
                        if (sp.window && !((end - dur) < sp.t_end && sp.t_start < end)) continue;
                        if (t < b.N && ((vis[t >> 5] >> (t & 31)) & 1u)) hit = true;
                    }
                } else if (sid >= 2 && sid - 2 < blk.C) {
                    const uint32_t c = sid - 2;
                    const glint_ctf_meta &m = blk.ctfs[c];
                    const uint32_t kb = m.key_bit / 8;
                    n = blk.count[u];
                    const uint8_t *base =
                        blk.keys + blk.byte_index[c] + (unsigned long long)(blk.first[u] - blk.key_index[c]) * kb;
                    const uint8_t *kend = blk.keys + blk.key_bytes;
                    for (uint32_t j = 0; j < n && !hit; ++j) {
                        unsigned __int128 v = load_key(base + (size_t)j * kb, kb, kend);
                        v >>= m.mbr_bit;
                        const uint32_t end = (uint32_t)(v & ((1ull << m.end_bit) - 1)) + blk.end_time_min;
                        v >>= m.end_bit;
                        const uint32_t dur = (uint32_t)(v & ((1ull << m.duration_bit) - 1));
                        v >>= m.duration_bit;
                        const uint32_t t = (uint32_t)(v & ((1ull << m.id_bit) - 1));
                        ++keys;
                        if (sp.window && !((end - dur) < sp.t_end && sp.t_start < end)) continue;
                        if (t < b.N && ((vis[t >> 5] >> (t & 31)) & 1u)) hit = true;
                    }
                }
            }
            found = __any_sync(0xffffffffu, hit);
        }
        for (int o = 16; o > 0; o >>= 1) keys += __shfl_down_sync(0xffffffffu, keys, o);
        if (lane == 0) {
            if (keys) atomicAdd(&b.scanned[s], keys);
            if (found) {
                const uint32_t idx = atomicAdd(&b.counts[s], 1u);
                if (idx < b.N) b.lists[((size_t)s * 2 + (sp.cur ^ 1u)) * b.N + idx] = u;
            }
        }
    }
}

/* the objects a pull hop reached join the reached set of pull slot blockIdx.y */
__global__ void k_serve_mark(HopArgs b) {
    const uint32_t s = b.active[blockIdx.y];
    const uint32_t n = min(b.counts[s], b.N);
    const uint32_t *next = b.lists + ((size_t)s * 2 + (b.param[s].cur ^ 1u)) * b.N;
    uint32_t *vis = b.visited + (size_t)s * b.words;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t u = next[i];
        atomicOr(&vis[u >> 5], 1u << (u & 31));
    }
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
    uint64_t reached = 0; /* seeds and every hop's new objects so far */
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
    uint32_t *front = nullptr;
    unsigned long long *pprefix = nullptr; /* pull slots' items (their unreached objects), prefix sums */
    unsigned int *ucount = nullptr;        /* [slot] unreached objects listed */
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
                  v->rscan, v->rel, v->rel_off, v->front, v->pprefix, v->ucount};
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
    A((void **)&v->front, sizeof(uint32_t) * S);
    A((void **)&v->pprefix, sizeof(unsigned long long) * (S + 1));
    A((void **)&v->ucount, sizeof(unsigned int) * S);
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
    a.front = v->front;
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
        for (uint32_t k : admitted) v->state[k].frontier = v->state[k].reached = cnt[k];
    }

    /* one hop for every active slot, over the kept blocks that can hold a
     * key inside its window: a key of a block ends at most at end_time_max
     * and starts no earlier than start_min, and it counts when
     * start < t_end and t_start < end */
    std::vector<uint32_t> act, rel, front;
    std::vector<uint32_t> rel_off(1, 0);
    std::vector<unsigned long long> prefix(1, 0), pprefix(1, 0);
    /* frontier walks first, then the pull slots (their frontier reaches at
     * least as many objects as are left) */
    std::vector<uint32_t> order;
    for (int pass = 0; pass < 2; ++pass)
        for (uint32_t k = 0; k < v->slots; ++k) {
            const SlotState &st = v->state[k];
            if (!st.busy || st.hop >= st.hops) continue;
            const bool pull = (uint64_t)st.frontier >= (uint64_t)N - st.reached;
            if (pull == (pass == 1)) order.push_back(k);
        }
    uint32_t n_push = 0;
    for (uint32_t k : order) {
        const SlotState &st = v->state[k];
        const bool pull = (uint64_t)st.frontier >= (uint64_t)N - st.reached;
        act.push_back(k);
        front.push_back(st.frontier);
        const SlotParam &sp = v->hparam[k];
        uint32_t nrel = 0;
        for (uint32_t i = 0; i < nb; ++i) {
            const StoreBlock &b = c->ctbs[i];
            if (sp.window && b.spans_known && !(b.start_min < sp.t_end && sp.t_start < b.end_time_max)) continue;
            rel.push_back(i);
            ++nrel;
        }
        rel_off.push_back((uint32_t)rel.size());
        if (pull) {
            pprefix.push_back(pprefix.back() + ((uint64_t)N - st.reached));
        } else {
            prefix.push_back(prefix.back() + (unsigned long long)st.frontier * nrel);
            ++n_push;
        }
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
        cudaMemcpyAsync(v->front, front.data(), sizeof(uint32_t) * front.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->prefix, prefix.data(), sizeof(unsigned long long) * prefix.size(), cudaMemcpyHostToDevice,
                        s);
        cudaMemcpyAsync(v->pprefix, pprefix.data(), sizeof(unsigned long long) * pprefix.size(),
                        cudaMemcpyHostToDevice, s);
        if (!rel.empty())
            cudaMemcpyAsync(v->rel, rel.data(), sizeof(uint32_t) * rel.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(v->rel_off, rel_off.data(), sizeof(uint32_t) * rel_off.size(), cudaMemcpyHostToDevice, s);
        for (uint32_t k : act) cudaMemsetAsync(v->counts + k, 0, sizeof(uint32_t), s);
        a.A = n_push;
        const unsigned long long items = prefix.back();
        if (items) k_serve_hop<<<grid_for((items + 31) / 32, kHopThreads / 32, 152u * 8u), kHopThreads, 0, s>>>(a);
        const uint32_t n_pull = (uint32_t)act.size() - n_push;
        if (n_pull) {
            HopArgs b = a;
            b.active = v->active + n_push;
            b.rel_off = v->rel_off + n_push;
            b.prefix = v->pprefix;
            b.A = n_pull;
            for (uint32_t i = n_push; i < act.size(); ++i) cudaMemsetAsync(v->ucount + act[i], 0, sizeof(unsigned), s);
            const uint32_t nw = (N + 31) / 32;
            k_serve_unvisited<<<dim3(std::min<uint32_t>((nw + 255) / 256, 1024u), n_pull), 256, 0, s>>>(b, v->ucount);
            const unsigned long long objs = pprefix.back();
            if (objs) k_serve_pull<<<grid_for(objs, 8, 152u * 16u), 256, 0, s>>>(b);
            k_serve_mark<<<dim3(64, n_pull), 256, 0, s>>>(b);
        }
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
            st.reached += got;
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
        v->rel = v->rel_off = v->front = nullptr;
        v->pprefix = nullptr;
        v->ucount = nullptr;
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
