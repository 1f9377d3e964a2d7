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
 * Device form: a stamp byte per bucket says empty or committed, and a bit per
 * 128-byte line of the table says that the insert placed a pair in it this
 * step, so the scan reads one byte per bucket and the 32-byte records only of
 * committed entries and of lines that received a pair.  Pass 1 (32 consecutive buckets
 * per warp and round) finalises entries inserted this step, removes expired
 * entries that are too short, marks the ones to report and counts them per
 * 8192-bucket tile; an exclusive scan gives every tile its offset; pass 2
 * visits only tiles with reports and writes them in bucket order into the
 * device meeting log, then removes those entries.
 */
#include "glint_internal.cuh"

namespace glint {

constexpr int kIdThreads = 256;
constexpr uint32_t kIdWarpSpan = 1024;                      /* buckets per warp, 32 rounds of 32 */
constexpr uint32_t kIdTile = (kIdThreads / 32) * kIdWarpSpan; /* 8192 buckets per block */
constexpr uint8_t kStampEmit = 4;

/* Pass 1.  Warp w of a block walks buckets tile + w*1024 + round*32 + lane,
 * so each round reads 32 consecutive stamps and, where needed, 32
 * consecutive records: the records of one round share DRAM lines.  The
 * warp's 1024 stamps are staged in shared memory with one coalesced load, and
 * the records of kIdIlp rounds are requested before any is used. */
constexpr int kIdIlp = 4;

__global__ void __launch_bounds__(kIdThreads) k_expire_count(uint8_t *__restrict__ stamp,
                                                             uint32_t *__restrict__ newline,
                                                             TRec *__restrict__ tab, uint64_t B, uint32_t min_plus1,
                                                             uint32_t *__restrict__ tile_cnt,
                                                             const float2 *__restrict__ fpos, uint32_t N,
                                                             DevCounters *cnt) {
    __shared__ uint32_t red[3][kIdThreads / 32];
    __shared__ __align__(16) uint8_t sst[kIdThreads / 32][kIdWarpSpan];
    __shared__ uint32_t snl[kIdThreads / 32][kIdWarpSpan / 128];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint64_t wbase = (uint64_t)blockIdx.x * kIdTile + (uint64_t)wid * kIdWarpSpan;
    const uint32_t cur_time = cnt->step_time, st_now = cnt->step_tag;
    /* stamps and new-line words are allocated to a whole number of tiles */
    const uint4 *src = reinterpret_cast<const uint4 *>(stamp + wbase);
    uint4 *dst = reinterpret_cast<uint4 *>(sst[wid]);
    dst[lane] = src[lane];
    dst[lane + 32] = src[lane + 32];
    if (lane < (int)(kIdWarpSpan / 128)) {
        /* the warp's lines filled this step; cleared for the next step */
        snl[wid][lane] = newline[(wbase >> 7) + lane];
        newline[(wbase >> 7) + lane] = 0;
    }
    __syncwarp();
    uint32_t emit = 0, taken = 0, active = 0;
    for (uint32_t r0 = 0; r0 < kIdWarpSpan / 32; r0 += kIdIlp) {
        uint8_t sv[kIdIlp];
        bool need[kIdIlp];
        ulonglong2 rec[kIdIlp];
#pragma unroll
        for (int u = 0; u < kIdIlp; ++u) {
            const uint32_t off = (r0 + u) * 32 + lane;
            sv[u] = wbase + off < B ? sst[wid][off] : kStampEmpty;
            need[u] = sv[u] != kStampEmpty || (wbase + off < B && ((snl[wid][off >> 7] >> ((off >> 2) & 31)) & 1u));
            if (need[u]) rec[u] = *reinterpret_cast<const ulonglong2 *>(&tab[wbase + off]);
        }
#pragma unroll
        for (int u = 0; u < kIdIlp; ++u) {
            if (!need[u]) continue;
            const uint64_t b = wbase + (r0 + u) * 32 + lane;
            TRec &r = tab[b];
            if (sv[u] == kStampEmpty) {
                /* a slot of a line that received a pair this step: empty, or
                 * the pair (key word with kNewFlag).  Its start is now and its
                 * box that of its two points (geometry.cu:481-489). */
                if (rec[u].x == kEmptyW0 || !(rec[u].x & kNewFlag)) continue;
                ++taken;
                ++active;
                const unsigned long long pw = rec[u].x & kPairMask;
                const uint32_t pa = pair_a(pw), pb = pair_b(pw);
                TRec nr;
                nr.w0 = pw;
                nr.w1 = ((unsigned long long)st_now << 32) | cur_time;
                if (pa < N && pb < N) {
                    const float2 A = fpos[pa], Bp = fpos[pb];
                    nr.mbr[0] = min(fenc(A.x), fenc(Bp.x));
                    nr.mbr[1] = min(fenc(A.y), fenc(Bp.y));
                    nr.mbr[2] = max(fenc(A.x), fenc(Bp.x));
                    nr.mbr[3] = max(fenc(A.y), fenc(Bp.y));
                } else {
                    atomicOr(&cnt->error_flags, GLINT_EF_DUPLICATE_NEW);
                    nr.mbr[0] = nr.mbr[1] = nr.mbr[2] = nr.mbr[3] = 0;
                }
                r = nr;
                stamp[b] = kStampOld;
                continue;
            }
            ++taken;
            const unsigned long long w1 = rec[u].y;
            if ((uint32_t)(w1 >> 32) == st_now) {
                ++active;
                continue;
            }
            const uint32_t start = (uint32_t)w1;
            if (cur_time - start >= min_plus1) {
                ++emit;
                stamp[b] = kStampEmit;
            } else {
                *reinterpret_cast<ulonglong2 *>(&r) = make_ulonglong2(kEmptyW0, 0ull);
                stamp[b] = kStampEmpty;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        emit += __shfl_down_sync(0xffffffffu, emit, o);
        taken += __shfl_down_sync(0xffffffffu, taken, o);
        active += __shfl_down_sync(0xffffffffu, active, o);
    }
    if (lane == 0) {
        red[0][wid] = emit;
        red[1][wid] = taken;
        red[2][wid] = active;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t e = 0, t = 0, a = 0;
        for (int i = 0; i < kIdThreads / 32; ++i) {
            e += red[0][i];
            t += red[1][i];
            a += red[2][i];
        }
        tile_cnt[blockIdx.x] = e;
        if (t) atomicAdd(&cnt->taken, (unsigned long long)t);
        if (a) atomicAdd(&cnt->active, a);
    }
}

/* Pass 2: the reports of tiles that have any, in bucket order (warps in
 * order, rounds in order, lanes in order), into the meeting log */
__global__ void __launch_bounds__(kIdThreads) k_expire_emit(uint8_t *__restrict__ stamp, TRec *__restrict__ tab,
                                                            uint64_t B,
                                                            const uint32_t *__restrict__ tile_cnt,
                                                            const uint32_t *__restrict__ tile_off,
                                                            glint_meeting *__restrict__ log, uint64_t log_cap,
                                                            const DevCounters *cnt) {
    if (tile_cnt[blockIdx.x] == 0) return; /* uniform per block */
    __shared__ uint32_t ws[kIdThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint64_t wbase = (uint64_t)blockIdx.x * kIdTile + (uint64_t)wid * kIdWarpSpan;
    uint32_t mine = 0;
    for (uint32_t round = 0; round < kIdWarpSpan / 32; ++round) {
        const uint64_t b = wbase + round * 32 + lane;
        if (b < B && stamp[b] == kStampEmit) ++mine;
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if (lane == 0) ws[wid] = mine;
    __syncthreads();
    uint32_t pos = tile_off[blockIdx.x];
    for (int w = 0; w < wid; ++w) pos += ws[w];
    if (mine == 0) return;
    const unsigned long long head = cnt->log_head;
    const uint32_t cur_time = cnt->step_time;
    for (uint32_t round = 0; round < kIdWarpSpan / 32; ++round) {
        const uint64_t b = wbase + round * 32 + lane;
        const bool e = b < B && stamp[b] == kStampEmit;
        const unsigned m = __ballot_sync(0xffffffffu, e);
        if (e) {
            TRec &r = tab[b];
            const unsigned long long w0 = r.w0;
            const uint4 mb = *reinterpret_cast<const uint4 *>(r.mbr);
            glint_meeting out;
            out.pid1 = pair_a(w0);
            out.pid2 = pair_b(w0);
            out.start = (uint32_t)r.w1;
            out.end = cur_time - 1;
            out.mbr[0] = fdec(mb.x);
            out.mbr[1] = fdec(mb.y);
            out.mbr[2] = fdec(mb.z);
            out.mbr[3] = fdec(mb.w);
            log[(head + pos + __popc(m & ((1u << lane) - 1u))) % log_cap] = out;
            *reinterpret_cast<ulonglong2 *>(&r) = make_ulonglong2(kEmptyW0, 0ull);
            stamp[b] = kStampEmpty;
        }
        pos += __popc(m);
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

uint64_t identify_tiles(uint64_t B) { return (B + kIdTile - 1) / kIdTile; }

cudaError_t launch_identify(glint_ctx *c, uint32_t cur_time) {
    (void)cur_time;
    cudaStream_t s = c->stream;
    const uint64_t tiles = identify_tiles(c->B);
    const uint32_t min_plus1 = c->cfg.min_meet_time + 1;
    k_expire_count<<<(unsigned)tiles, kIdThreads, 0, s>>>(c->d_stamp, c->d_newline, c->d_tab, c->B, min_plus1,
                                                          c->d_tile_cnt,
                                                          c->d_fpos, c->N, c->d_cnt);
    scan_u32(c->d_tile_cnt, c->d_tile_off, tiles, c->d_scan_tmp, s);
    k_expire_emit<<<(unsigned)tiles, kIdThreads, 0, s>>>(c->d_stamp, c->d_tab, c->B, c->d_tile_cnt, c->d_tile_off,
                                                         c->d_log, c->log_cap, c->d_cnt);
    k_identify_advance<<<1, 1, 0, s>>>(c->d_tile_off, tiles, c->log_cap, c->d_cnt);
    return cudaGetLastError();
}

} // namespace glint
