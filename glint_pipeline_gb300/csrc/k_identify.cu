/*
 * k_identify.cu -- stage (d) part 2: expire finished meetings and emit the
 * ones that lasted long enough.
 *
 * Reference: update_meetings_unit (tracing/meeting.cpp:32-76) scans every
 * bucket: an entry touched this step (end == cur_time) is active; any other
 * entry is removed, and reported first when cur_time - start >=
 * min_meet_time + 1.  With one thread the reports come out in bucket order
 * (batch_meet, tracing/meeting.cpp:11-24).
 *
 * Device form: a stamp byte per bucket says empty / touched at this step /
 * touched at the previous step / inserted this step, so the scan reads one
 * byte per bucket and touches the 32-byte record only for entries that
 * change.  Pass 1 counts the emissions of each 4096-bucket tile, an exclusive
 * scan gives every tile its offset, and pass 2 writes the meetings in bucket
 * order into the device log, finalises this step's new entries (start = now,
 * f32 box of the pair's two points, geometry.cu:481-489) and clears the
 * expired ones.
 */
#include "glint_internal.cuh"

namespace glint {

constexpr int kIdThreads = 1024;
constexpr int kIdItems = 4;
constexpr uint32_t kIdTile = kIdThreads * kIdItems;

__device__ inline uint32_t block_scan_excl(uint32_t v, uint32_t *ws, uint32_t &total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    uint32_t pre = (wid ? ws[wid - 1] : 0u) + x - v;
    total = ws[(blockDim.x >> 5) - 1];
    __syncthreads();
    return pre;
}

__global__ void __launch_bounds__(kIdThreads) k_identify_count(const uint8_t *__restrict__ stamp,
                                                               const TRec *__restrict__ tab, uint64_t B,
                                                               uint8_t st_now, uint32_t cur_time, uint32_t min_plus1,
                                                               uint32_t *__restrict__ tile_cnt, DevCounters *cnt) {
    __shared__ uint32_t ws[32];
    const uint64_t base = (uint64_t)blockIdx.x * kIdTile + (uint64_t)threadIdx.x * kIdItems;
    uint32_t emit = 0, taken = 0, active = 0;
    uint32_t st4 = 0;
    if (base + kIdItems <= B) st4 = *reinterpret_cast<const uint32_t *>(stamp + base);
    else
        for (int k = 0; k < kIdItems; ++k)
            if (base + k < B) st4 |= (uint32_t)stamp[base + k] << (8 * k);
#pragma unroll
    for (int k = 0; k < kIdItems; ++k) {
        const uint8_t sv = (uint8_t)(st4 >> (8 * k));
        if (sv == kStampEmpty) continue;
        ++taken;
        if (sv == kStampNew || sv == st_now) {
            ++active;
            continue;
        }
        const uint32_t start = (uint32_t)tab[base + k].w1;
        if (cur_time - start >= min_plus1) ++emit;
    }
    uint32_t tot_e, tot_t, tot_a;
    block_scan_excl(emit, ws, tot_e);
    block_scan_excl(taken, ws, tot_t);
    block_scan_excl(active, ws, tot_a);
    if (threadIdx.x == 0) {
        tile_cnt[blockIdx.x] = tot_e;
        if (tot_t) atomicAdd(&cnt->taken, (unsigned long long)tot_t);
        if (tot_a) atomicAdd(&cnt->active, tot_a);
    }
}

__global__ void __launch_bounds__(kIdThreads) k_identify_write(uint8_t *__restrict__ stamp, TRec *__restrict__ tab,
                                                               uint64_t B, uint8_t st_now, uint32_t cur_time,
                                                               uint32_t min_plus1, const uint32_t *__restrict__ tile_off,
                                                               const double2 *__restrict__ pts,
                                                               glint_meeting *__restrict__ log, uint64_t log_cap,
                                                               uint32_t N, DevCounters *cnt) {
    __shared__ uint32_t ws[32];
    const uint64_t base = (uint64_t)blockIdx.x * kIdTile + (uint64_t)threadIdx.x * kIdItems;
    uint32_t st4 = 0;
    if (base + kIdItems <= B) st4 = *reinterpret_cast<const uint32_t *>(stamp + base);
    else
        for (int k = 0; k < kIdItems; ++k)
            if (base + k < B) st4 |= (uint32_t)stamp[base + k] << (8 * k);
    uint32_t emit_mask = 0;
    uint32_t starts[kIdItems];
#pragma unroll
    for (int k = 0; k < kIdItems; ++k) {
        starts[k] = 0;
        const uint8_t sv = (uint8_t)(st4 >> (8 * k));
        if (sv == kStampEmpty || sv == st_now || sv == kStampNew) continue;
        starts[k] = (uint32_t)tab[base + k].w1;
        if (cur_time - starts[k] >= min_plus1) emit_mask |= 1u << k;
    }
    uint32_t tot;
    uint32_t pos = block_scan_excl((uint32_t)__popc(emit_mask), ws, tot) + tile_off[blockIdx.x];
    const unsigned long long head = cnt->log_head;
    uint32_t new_st4 = st4;
    bool changed = false;
#pragma unroll
    for (int k = 0; k < kIdItems; ++k) {
        const uint8_t sv = (uint8_t)(st4 >> (8 * k));
        const uint64_t slot = base + k;
        if (sv == kStampEmpty || sv == st_now) continue;
        changed = true;
        if (sv == kStampNew) {
            /* finalise an entry inserted this step */
            const unsigned long long key = tab[slot].w0 & kKeyMask;
            uint32_t pa, pb;
            cantor_inverse(key, pa, pb);
            if (pa >= N || pb >= N) {
                atomicOr(&cnt->error_flags, GLINT_EF_DUPLICATE_NEW);
                pa = pb = 0;
            }
            const double2 A = pts[pa], Bp = pts[pb];
            const float ax = (float)A.x, ay = (float)A.y, bx = (float)Bp.x, by = (float)Bp.y;
            TRec r;
            r.w0 = key;
            r.w1 = cur_time;
            r.mbr[0] = min(fenc(ax), fenc(bx));
            r.mbr[1] = min(fenc(ay), fenc(by));
            r.mbr[2] = max(fenc(ax), fenc(bx));
            r.mbr[3] = max(fenc(ay), fenc(by));
            tab[slot] = r;
            new_st4 = (new_st4 & ~(0xffu << (8 * k))) | ((uint32_t)st_now << (8 * k));
            continue;
        }
        /* expire */
        if (emit_mask & (1u << k)) {
            const unsigned long long key = tab[slot].w0;
            uint32_t pa, pb;
            cantor_inverse(key, pa, pb);
            const uint4 m = *reinterpret_cast<const uint4 *>(tab[slot].mbr);
            glint_meeting out;
            out.pid1 = pa;
            out.pid2 = pb;
            out.start = starts[k];
            out.end = cur_time - 1;
            out.mbr[0] = fdec(m.x);
            out.mbr[1] = fdec(m.y);
            out.mbr[2] = fdec(m.z);
            out.mbr[3] = fdec(m.w);
            log[(head + pos) % log_cap] = out;
            ++pos;
        }
        tab[slot].w0 = kEmptyKey;
        new_st4 &= ~(0xffu << (8 * k));
    }
    if (changed) {
        if (base + kIdItems <= B) *reinterpret_cast<uint32_t *>(stamp + base) = new_st4;
        else
            for (int k = 0; k < kIdItems; ++k)
                if (base + k < B) stamp[base + k] = (uint8_t)(new_st4 >> (8 * k));
    }
}

__global__ void k_identify_advance(const uint32_t *__restrict__ tile_off, uint64_t tiles, uint64_t log_cap,
                                   DevCounters *cnt) {
    const uint32_t total = tile_off[tiles];
    cnt->meetings = total;
    cnt->log_step_begin = cnt->log_head;
    cnt->log_head += total;
    if (total > log_cap) atomicOr(&cnt->error_flags, GLINT_EF_LOG_OVERFLOW);
}

cudaError_t launch_identify(glint_ctx *c, uint32_t cur_time) {
    cudaStream_t s = c->stream;
    const uint64_t tiles = (c->B + kIdTile - 1) / kIdTile;
    const uint8_t st_now = stamp_of(c->step_index);
    const uint32_t min_plus1 = c->cfg.min_meet_time + 1;
    k_identify_count<<<(unsigned)tiles, kIdThreads, 0, s>>>(c->d_stamp, c->d_tab, c->B, st_now, cur_time, min_plus1,
                                                            c->d_tile_cnt, c->d_cnt);
    scan_u32(c->d_tile_cnt, c->d_tile_off, tiles, c->d_scan_tmp, s);
    k_identify_write<<<(unsigned)tiles, kIdThreads, 0, s>>>(c->d_stamp, c->d_tab, c->B, st_now, cur_time, min_plus1,
                                                            c->d_tile_off, c->d_pts, c->d_log, c->log_cap, c->N, c->d_cnt);
    k_identify_advance<<<1, 1, 0, s>>>(c->d_tile_off, tiles, c->log_cap, c->d_cnt);
    return cudaGetLastError();
}

uint64_t identify_tiles(uint64_t B) { return (B + kIdTile - 1) / kIdTile; }

} // namespace glint
