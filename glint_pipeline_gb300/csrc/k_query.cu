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
 * the record of occupied buckets (its tag says whether the last step touched
 * it), and counts matching
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
    uint8_t st;              /* tag of entries touched at the last step */
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
    if (r.w0 == kEmptyW0 || (r.w0 & kNewFlag) || rec_tag(r) != a.st) return 0;
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
        if ((uint8_t)(w[k >> 2] >> (8 * (k & 3))) != kStampOld || base + k >= a.B) continue;
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
    if (serve_only_refused(c, "active search")) return GLINT_ERR_STATE;
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

/* exclusive scan of n (<= kNaMaxTiles) values by one block, no scratch;
 * out[n] receives the total, so out has n + 1 words and in only n are read */
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
    if (threadIdx.x == 0) out[n] = carry;
}

/* looks up the scratch address on the current device; run by every
 * glint_create, so a context created after a device reset sees the array's
 * address in the device's new CUDA context */
cudaError_t noalloc_setup(int device) {
    if (device < 0 || device >= kNaMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    void *p = nullptr;
    g_na_status[device] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    g_na_ptr[device] = g_na_status[device] == cudaSuccess ? static_cast<uint32_t *>(p) : nullptr;
    g_na_done[device] = true;
    return g_na_status[device];
}

} // namespace glint

extern "C" glint_status glint_active_search_noalloc(glint_ctx *c, const uint32_t *d_pids, uint32_t npids,
                                                    glint_search_info *d_out, uint64_t cap, uint64_t *d_n) {
    if (!c || (npids && !d_pids) || (cap && !d_out) || !d_n) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "active search")) return GLINT_ERR_STATE;
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
        k_scan_one_block<<<1, 1024, 0, s>>>(in, o, m);
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

