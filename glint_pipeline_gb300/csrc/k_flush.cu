/*
 * k_flush.cu -- stage (e): the key-value + bitmap store.
 *
 * Key generation (every step, after identify): each meeting identified this
 * step whose box lies inside the map becomes two keys, as the report branch
 * of cuda_identify_meetings (cuda/geometry.cu:665-734):
 *   key = [sid:12][pid:26][target:26][end - start:32][end - end_time_min:32]
 * one per direction, with its f32 box; per object, a key count
 * (same_pid_count) and the union of its boxes in the reference's fixed-point
 * form (float_to_uint, cuda/cuda_util.cuh:116-120).  A meeting longer than
 * max_meet_time marks both objects oversize.
 *
 * Flush (cuda/geometry.cu:1752-2135), restated stage by stage:
 *   set_oid            objects' mean position key, area cut -> oversize
 *   partition          keys of oversize objects go to the oversize buffer
 *   STR                stable sort of objects by mean x, then by mean y
 *                      inside split_num x-slices; make_sid numbers the
 *                      split_num^2 cells 2.. (0: no keys, 1: oversize)
 *   key sort           the CTF keys carry their sid; both parts sorted
 *   get_CTF_capacity, cuda_get_limit (with its lane-32..63 quirk, below),
 *   CTF::get_ctf_bits (host, tracing/step_merge.cpp:140-186),
 *   cuda_write_bitmap, write_key_and_mbr (packing into key_bit/8 bytes),
 *   get_o_limit, cuda_write_o_bitmap for the oversize buffer.
 *
 * Device form of the sorts (the reference uses thrust): the STR sorts are
 * stable LSD radix sorts (k_sort.cu).  The key sorts exploit the key layout:
 * keys group by (part, sid, pid), so objects are radix-sorted by that triple,
 * each object's keys get a contiguous segment (a scan of the key counts), the
 * keys are scattered into their segments and each segment (a few keys, at
 * most kSegBlockMax) is sorted by a warp or a block.
 *
 * The reference's cuda_get_limit and get_o_limit fold a 1024-entry shared
 * reduction down to 64 partial results and then shuffle-reduce only the
 * first 32: a key at offset o of its range contributes only if
 * o mod 64 < 32.  The CTF boxes and start times computed here follow that
 * rule, because bit widths, bitmaps and packed keys depend on them.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "glint_internal.cuh"
#include "store_codec.cuh"

namespace glint {


constexpr int kOidBit = 26;            /* util/util.h:49 */
constexpr int kSidShift = 2 * kOidBit + 64;
constexpr int kPidShift = kOidBit + 64;
constexpr uint32_t kBitEdge = 256;     /* DEFAULT_bitmap_edge, util/util.h:47 */
constexpr uint64_t kBitCount = (uint64_t)kBitEdge * kBitEdge;
constexpr uint32_t kSegWarpMax = 256;
constexpr uint32_t kSegBlockMax = 8192;
constexpr unsigned long long kGroupNone = 2ull << 40;

typedef unsigned __int128 u128;

__device__ inline uint32_t key_oid(u128 k) { return (uint32_t)(k >> kPidShift) & ((1u << kOidBit) - 1); }
__device__ inline uint32_t key_sid(u128 k) { return (uint32_t)(k >> kSidShift) & 0xfffu; }

/* float_to_uint (cuda/cuda_util.cuh:116-120) */
__device__ inline uint32_t f2u_coord(float xy) { return __float2uint_rz(__fmul_rn(__fadd_rn(xy, 180.0f), 100000.0f)); }
/* uint_to_float (cuda/cuda_util.cuh:122-126) */
__device__ inline float u2f_coord(uint32_t f) { return __fsub_rn(__fdiv_rn(__uint2float_rn(f), 100000.0f), 180.0f); }

struct KeyArgs {
    u128 *keys;
    float4 *boxes;
    uint64_t cap;
    uint32_t *same;
    uint4 *obox;
    uint16_t *sids;
    double map[4];
    uint32_t max_meet;
};

/* the meetings this step wrote to the log become keys */
__global__ void __launch_bounds__(256) k_keys_append(const glint_meeting *__restrict__ log, uint64_t log_cap,
                                                     KeyArgs a, DevCounters *cnt) {
    const uint32_t total = cnt->meetings;
    const unsigned long long begin = cnt->log_step_begin;
    const uint32_t end_time_min = cnt->end_time_min;
    const int lane = threadIdx.x & 31;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 - lane < total; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0;
        glint_meeting m;
        bool keep = false;
        if (i < total) {
            m = log[(begin + i) % log_cap];
            /* box_contain (cuda/geometry.cu:53-58, 667-670) */
            keep = (double)m.mbr[0] >= a.map[0] && (double)m.mbr[2] <= a.map[2] && (double)m.mbr[1] >= a.map[1] &&
                   (double)m.mbr[3] <= a.map[3];
            if (!keep) atomicAdd(&cnt->keys_outside, 1u);
        }
        /* two keys per kept meeting, reserved once per warp */
        const unsigned km = __ballot_sync(0xffffffffu, keep);
        unsigned long long wbase = 0;
        if (km) {
            const int leader = __ffs(km) - 1;
            if (lane == leader) wbase = atomicAdd(&cnt->kv_count, 2ull * __popc(km));
            wbase = __shfl_sync(0xffffffffu, wbase, leader);
        }
        if (!keep) continue;
        const uint32_t duration = m.end - m.start;
        uint32_t pid = m.pid1, target = m.pid2;
        if (duration > a.max_meet) {
            atomicAdd(&cnt->oversize_oid_count, 1u);
            a.sids[pid] = 1;
            a.sids[target] = 1;
        }
        const unsigned long long idx = wbase + 2ull * __popc(km & ((1u << lane) - 1u));
        if (idx + 2 > a.cap) {
            atomicOr(&cnt->error_flags, GLINT_EF_KV_OVERFLOW);
            continue;
        }
        const float4 box = make_float4(m.mbr[0], m.mbr[1], m.mbr[2], m.mbr[3]);
        const uint32_t l0 = f2u_coord(box.x), l1 = f2u_coord(box.y), h0 = f2u_coord(box.z), h1 = f2u_coord(box.w);
        for (int k = 0; k < 2; ++k) {
            if (k == 1) {
                const uint32_t t = pid;
                pid = target;
                target = t;
            }
            a.keys[idx + k] = ((u128)pid << kPidShift) + ((u128)target << 64) + ((u128)duration << 32) +
                              (u128)(uint32_t)(m.end - end_time_min);
            a.boxes[idx + k] = box;
            atomicAdd(&a.same[pid], 1u); /* objects with keys are counted at the flush */
            uint32_t *o = reinterpret_cast<uint32_t *>(&a.obox[pid]);
            atomicMin(&o[0], l0);
            atomicMin(&o[1], l1);
            atomicMax(&o[2], h0);
            atomicMax(&o[3], h1);
        }
    }
}

__global__ void k_init_obox(uint4 *obox, uint32_t N) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        obox[i] = make_uint4(100000000u, 100000000u, 0u, 0u); /* cuda_init_o_boxs (:1254-1263) */
}

/* set_oid (cuda/geometry.cu:739-769); also records which objects' keys go to
 * the oversize buffer (partition, :1784-1797) */
__global__ void __launch_bounds__(256) k_set_oid(uint32_t N, const uint32_t *__restrict__ same,
                                                 const uint4 *__restrict__ obox, uint16_t *__restrict__ sids,
                                                 double dprob, uint32_t *__restrict__ oids,
                                                 unsigned long long *__restrict__ mid, uint8_t *__restrict__ over,
                                                 DevCounters *cnt) {
    uint32_t with_keys = 0;
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x) {
        oids[id] = id;
        unsigned long long m = 0;
        if (same[id] >= 1) {
            ++with_keys;
            const uint4 o = obox[id];
            const float low0 = u2f_coord(o.x), high0 = u2f_coord(o.z), low1 = u2f_coord(o.y), high1 = u2f_coord(o.w);
            const float area = __fmul_rn(__fsub_rn(high1, low1), __fsub_rn(high0, low0));
            if ((double)area > dprob) {
                atomicAdd(&cnt->oversize_oid_count, 1u);
                sids[id] = 1;
            } else {
                const uint32_t ave_mid0 = o.x / 2 + o.z / 2;
                const uint32_t ave_mid1 = o.w / 2 + o.w / 2; /* high[1] twice, as the reference */
                m = ((unsigned long long)ave_mid0 << 32) + ave_mid1;
            }
        }
        mid[id] = m;
        over[id] = 0; /* finalised by k_mark_over once every area cut is in */
    }
    /* sid_count: objects with at least one key in this window */
    with_keys = __reduce_add_sync(0xffffffffu, with_keys);
    if ((threadIdx.x & 31) == 0 && with_keys) atomicAdd(&cnt->sid_count, with_keys);
}

__global__ void k_mark_over(uint32_t N, const uint16_t *__restrict__ sids, uint8_t *__restrict__ over) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x)
        over[id] = sids[id] == 1 ? 1 : 0;
}

/* narrow_xy_to_y (:771-778) + the per-slice sort keys (:1881-1890): slice
 * index + 1 above the y half, 0 for the objects before the slices */
__global__ void k_str_slice_keys(unsigned long long *__restrict__ mid, uint32_t N, uint32_t zero_one, uint32_t x_part,
                                 uint32_t split) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x) {
        if (id < zero_one) {
            mid[id] = 0;
            continue;
        }
        uint32_t part = (id - zero_one) / x_part;
        if (part > split - 1) part = split - 1;
        mid[id] = ((unsigned long long)(part + 1) << 32) | (mid[id] & 0xffffffffull);
    }
}

/* make_sid (:780-796) */
__global__ void k_make_sid(const uint32_t *__restrict__ oids, uint32_t N, uint32_t zero_one, uint32_t x_part,
                           uint32_t split, uint16_t *__restrict__ sids) {
    const uint32_t part_key = x_part / split + 1;
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x) {
        if (id < zero_one) continue;
        const uint32_t xi = (id - zero_one) / x_part;
        const uint32_t yi = (id - zero_one - xi * x_part) / part_key;
        sids[oids[id]] = (uint16_t)(xi * split + yi + 2);
    }
}

/* object order of the key segments: (oversize part, sid, oid) */
__global__ void k_group_keys(uint32_t N, const uint32_t *__restrict__ same, const uint16_t *__restrict__ sids,
                             const uint8_t *__restrict__ over, unsigned long long *__restrict__ gk,
                             uint32_t *__restrict__ gv) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x) {
        unsigned long long k = kGroupNone;
        if (same[id]) {
            k = over[id] ? ((1ull << 40) | id) : (((unsigned long long)sids[id] << kOidBit) | id);
        }
        gk[id] = k;
        gv[id] = id;
    }
}

__global__ void k_group_counts(uint32_t N, const unsigned long long *__restrict__ gk, const uint32_t *__restrict__ gv,
                               const uint32_t *__restrict__ same, uint32_t *__restrict__ c) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        c[i] = gk[i] == kGroupNone ? 0u : same[gv[i]];
}

/* segment start of every object; the total of the CTF part */
__global__ void k_group_starts(uint32_t N, const unsigned long long *__restrict__ gk, const uint32_t *__restrict__ gv,
                               const uint32_t *__restrict__ start, uint32_t *__restrict__ seg_of,
                               unsigned long long *__restrict__ main_count) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        seg_of[gv[i]] = start[i];
        const bool is_main = gk[i] < (1ull << 40);
        const bool next_main = i + 1 < N && gk[i + 1] < (1ull << 40);
        if (is_main && !next_main) *main_count = start[i + 1];
        if (i == 0 && !is_main) *main_count = 0;
    }
}

/* an object's placement record for the key scatter: its segment start, its
 * sid and its oversize mark in 8 bytes, so that a key costs one random record
 * and one random cursor instead of four scattered per-object arrays */
__global__ void k_obj_place(uint32_t N, const uint32_t *__restrict__ seg_of, const uint16_t *__restrict__ sids,
                            const uint8_t *__restrict__ over, uint2 *__restrict__ place) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x)
        place[o] = make_uint2(seg_of[o], (uint32_t)sids[o] | ((uint32_t)over[o] << 16));
}

__global__ void k_key_scatter(const u128 *__restrict__ keys, const float4 *__restrict__ boxes, uint64_t n,
                              const uint2 *__restrict__ place, uint32_t *__restrict__ cur,
                              u128 *__restrict__ okeys, float4 *__restrict__ oboxes) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        u128 k = keys[i];
        const uint32_t oid = key_oid(k);
        const uint32_t slot = atomicAdd(&cur[oid], 1u);
        const uint2 pl = place[oid];
        /* write_sid_in_key (:798-806) for the CTF part */
        if (!(pl.y >> 16)) k = (k & (((u128)1 << kSidShift) - 1)) + ((u128)(pl.y & 0xffffu) << kSidShift);
        okeys[pl.x + slot] = k;
        oboxes[pl.x + slot] = boxes[i];
    }
}

__device__ inline bool u128_less(u128 a, u128 b) { return a < b; }

constexpr uint32_t kSegTinyMax = 8;
constexpr uint32_t kSegHalfMax = 16;

/* segments of 2..8 keys, one thread each: the 19-comparator sorting network
 * for eight elements over (key, box), padded with the largest key */
__global__ void __launch_bounds__(256) k_seg_sort_tiny(const unsigned long long *__restrict__ gk,
                                                       const uint32_t *__restrict__ gv,
                                                       const uint32_t *__restrict__ start,
                                                       const uint32_t *__restrict__ same, uint32_t N,
                                                       u128 *__restrict__ keys, float4 *__restrict__ boxes,
                                                       uint32_t *__restrict__ mid, unsigned int *n_mid,
                                                       uint32_t *__restrict__ large, unsigned int *n_large) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < N; g += gridDim.x * blockDim.x) {
        if (gk[g] == kGroupNone) continue;
        const uint32_t n = same[gv[g]];
        if (n > kSegTinyMax && n <= kSegHalfMax) {
            mid[atomicAdd(n_mid, 1u)] = g; /* k_seg_sort_half */
            continue;
        }
        if (n > kSegHalfMax) {
            large[atomicAdd(n_large, 1u)] = g; /* k_seg_sort_warp */
            continue;
        }
        if (n <= 1 || n > kSegTinyMax) continue;
        const uint32_t b = start[g];
        u128 k[kSegTinyMax];
        float4 x[kSegTinyMax];
#pragma unroll
        for (uint32_t i = 0; i < kSegTinyMax; ++i) {
            k[i] = i < n ? keys[b + i] : ~(u128)0;
            x[i] = i < n ? boxes[b + i] : make_float4(0, 0, 0, 0);
        }
#define GLINT_CE(i, j)                   \
    if (k[j] < k[i]) {                   \
        const u128 tk = k[i];            \
        k[i] = k[j];                     \
        k[j] = tk;                       \
        const float4 tx = x[i];          \
        x[i] = x[j];                     \
        x[j] = tx;                       \
    }
        GLINT_CE(0, 1) GLINT_CE(2, 3) GLINT_CE(4, 5) GLINT_CE(6, 7)
        GLINT_CE(0, 2) GLINT_CE(1, 3) GLINT_CE(4, 6) GLINT_CE(5, 7)
        GLINT_CE(1, 2) GLINT_CE(5, 6) GLINT_CE(0, 4) GLINT_CE(3, 7)
        GLINT_CE(1, 5) GLINT_CE(2, 6)
        GLINT_CE(1, 4) GLINT_CE(3, 6)
        GLINT_CE(2, 4) GLINT_CE(3, 5)
        GLINT_CE(3, 4)
#undef GLINT_CE
#pragma unroll
        for (uint32_t i = 0; i < kSegTinyMax; ++i)
            if (i < n) {
                keys[b + i] = k[i];
                boxes[b + i] = x[i];
            }
    }
}

/* segments of 9..16 keys, two per warp: a 16-lane bitonic sort in registers
 * (the shuffles stay inside each half of the warp) */
__global__ void __launch_bounds__(128) k_seg_sort_half(const uint32_t *__restrict__ mid,
                                                       const unsigned int *__restrict__ n_mid,
                                                       const uint32_t *__restrict__ gv,
                                                       const uint32_t *__restrict__ start,
                                                       const uint32_t *__restrict__ same, u128 *__restrict__ keys,
                                                       float4 *__restrict__ boxes) {
    const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
    const uint32_t total = *n_mid;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t p = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 2; p < total; p += 2 * warps) {
        const uint32_t i = p + half;
        uint32_t n = 0, b = 0;
        if (i < total) {
            const uint32_t g = mid[i];
            n = same[gv[g]];
            b = start[g];
        }
        u128 k = ~(u128)0;
        float4 bx = make_float4(0, 0, 0, 0);
        if ((uint32_t)hl < n) {
            k = keys[b + hl];
            bx = boxes[b + hl];
        }
        for (int kk = 2; kk <= 16; kk <<= 1) {
            for (int j = kk >> 1; j > 0; j >>= 1) {
                const unsigned long long lo = (unsigned long long)k, hi = (unsigned long long)(k >> 64);
                const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, j);
                const unsigned long long ohi = __shfl_xor_sync(0xffffffffu, hi, j);
                const float4 ob = make_float4(__shfl_xor_sync(0xffffffffu, bx.x, j),
                                              __shfl_xor_sync(0xffffffffu, bx.y, j),
                                              __shfl_xor_sync(0xffffffffu, bx.z, j),
                                              __shfl_xor_sync(0xffffffffu, bx.w, j));
                const u128 o = ((u128)ohi << 64) | olo;
                const bool up = (hl & kk) == 0;
                const bool lower = (hl & j) == 0;
                const bool take_min = lower == up;
                if (take_min ? (o < k) : (k < o)) {
                    k = o;
                    bx = ob;
                }
            }
        }
        if ((uint32_t)hl < n) {
            keys[b + hl] = k;
            boxes[b + hl] = bx;
        }
    }
}

/* one warp sorts segments of up to kSegWarpMax keys: in registers up to 32,
 * else a shared-memory bitonic sort of (key, index) */
__global__ void __launch_bounds__(128) k_seg_sort_warp(const uint32_t *__restrict__ large,
                                                       const unsigned int *__restrict__ n_large,
                                                       const uint32_t *__restrict__ gv,
                                                       const uint32_t *__restrict__ start,
                                                       const uint32_t *__restrict__ same,
                                                       u128 *__restrict__ keys, float4 *__restrict__ boxes,
                                                       uint32_t *__restrict__ big, unsigned int *n_big) {
    __shared__ u128 sk[4][kSegWarpMax];
    __shared__ uint16_t si[4][kSegWarpMax];
    __shared__ float4 sb[4][kSegWarpMax];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t total = *n_large;
    for (uint32_t li = blockIdx.x * 4 + w; li < total; li += gridDim.x * 4) {
        const uint32_t g = large[li];
        const uint32_t n = same[gv[g]];
        const uint32_t b = start[g];
        if (n > kSegWarpMax) {
            if (lane == 0) big[atomicAdd(n_big, 1u)] = g;
            continue;
        }
        if (n <= 32) {
            u128 k = ~(u128)0;
            float4 bx = make_float4(0, 0, 0, 0);
            if ((uint32_t)lane < n) {
                k = keys[b + lane];
                bx = boxes[b + lane];
            }
            for (int kk = 2; kk <= 32; kk <<= 1) {
                for (int j = kk >> 1; j > 0; j >>= 1) {
                    const unsigned long long lo = (unsigned long long)k, hi = (unsigned long long)(k >> 64);
                    const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, j);
                    const unsigned long long ohi = __shfl_xor_sync(0xffffffffu, hi, j);
                    const float4 ob = make_float4(__shfl_xor_sync(0xffffffffu, bx.x, j),
                                                  __shfl_xor_sync(0xffffffffu, bx.y, j),
                                                  __shfl_xor_sync(0xffffffffu, bx.z, j),
                                                  __shfl_xor_sync(0xffffffffu, bx.w, j));
                    const u128 o = ((u128)ohi << 64) | olo;
                    const bool up = (lane & kk) == 0;
                    const bool lower = (lane & j) == 0;
                    const bool take_min = lower == up;
                    const bool o_less = u128_less(o, k);
                    if (take_min ? o_less : u128_less(k, o)) {
                        k = o;
                        bx = ob;
                    }
                }
            }
            if ((uint32_t)lane < n) {
                keys[b + lane] = k;
                boxes[b + lane] = bx;
            }
            continue;
        }
        uint32_t P = 64;
        while (P < n) P <<= 1;
        for (uint32_t i = lane; i < P; i += 32) {
            sk[w][i] = i < n ? keys[b + i] : ~(u128)0;
            si[w][i] = (uint16_t)i;
            if (i < n) sb[w][i] = boxes[b + i];
        }
        __syncwarp();
        for (uint32_t kk = 2; kk <= P; kk <<= 1) {
            for (uint32_t j = kk >> 1; j > 0; j >>= 1) {
                for (uint32_t i = lane; i < P; i += 32) {
                    const uint32_t l = i ^ j;
                    if (l > i) {
                        const u128 x = sk[w][i], y = sk[w][l];
                        const bool up = (i & kk) == 0;
                        if ((y < x) == up) {
                            sk[w][i] = y;
                            sk[w][l] = x;
                            const uint16_t t = si[w][i];
                            si[w][i] = si[w][l];
                            si[w][l] = t;
                        }
                    }
                }
                __syncwarp();
            }
        }
        for (uint32_t i = lane; i < n; i += 32) {
            keys[b + i] = sk[w][i];
            boxes[b + i] = sb[w][si[w][i]];
        }
        __syncwarp();
    }
}

/* one block per segment of up to kSegBlockMax keys */
__global__ void __launch_bounds__(1024) k_seg_sort_block(const uint32_t *__restrict__ big,
                                                         const uint32_t *__restrict__ gv,
                                                         const uint32_t *__restrict__ start,
                                                         const uint32_t *__restrict__ same, u128 *__restrict__ keys,
                                                         float4 *__restrict__ boxes, float4 *__restrict__ tmp_boxes,
                                                         DevCounters *cnt, const unsigned int *n_big) {
    extern __shared__ unsigned char smem[];
    u128 *sk = reinterpret_cast<u128 *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sk + kSegBlockMax);
    const uint32_t nb = *n_big;
    for (uint32_t bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const uint32_t g = big[bi];
        const uint32_t n = same[gv[g]];
        const uint32_t b = start[g];
        if (n > kSegBlockMax) {
            if (threadIdx.x == 0) atomicOr(&cnt->error_flags, GLINT_EF_SEGMENT_TOO_LARGE);
            continue;
        }
        uint32_t P = 1024;
        while (P < n) P <<= 1;
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
            sk[i] = i < n ? keys[b + i] : ~(u128)0;
            si[i] = i;
        }
        __syncthreads();
        for (uint32_t kk = 2; kk <= P; kk <<= 1) {
            for (uint32_t j = kk >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                    const uint32_t l = i ^ j;
                    if (l > i) {
                        const u128 x = sk[i], y = sk[l];
                        const bool up = (i & kk) == 0;
                        if ((y < x) == up) {
                            sk[i] = y;
                            sk[l] = x;
                            const uint32_t t = si[i];
                            si[i] = si[l];
                            si[l] = t;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) tmp_boxes[b + i] = boxes[b + si[i]];
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            keys[b + i] = sk[i];
            boxes[b + i] = tmp_boxes[b + i];
        }
        __syncthreads();
    }
}

/* get_CTF_capacity (:808-818); the C counters are summed per block in
 * shared memory first (C <= 4096) */
__global__ void __launch_bounds__(256) k_ctf_capacity(const uint32_t *__restrict__ oids, uint32_t N,
                                                      uint32_t zero_one, const uint16_t *__restrict__ sids,
                                                      const uint32_t *__restrict__ same, uint32_t C,
                                                      uint32_t *__restrict__ cap, DevCounters *cnt) {
    __shared__ uint32_t part[4096];
    for (uint32_t i = threadIdx.x; i < C; i += blockDim.x) part[i] = 0;
    __syncthreads();
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x) {
        if (id < zero_one) continue;
        const uint32_t oid = oids[id];
        const uint32_t c = (uint32_t)sids[oid] - 2u;
        if (c < C) atomicAdd(&part[c], same[oid]);
        else atomicOr(&cnt->error_flags, GLINT_EF_STORE_DOMAIN);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < C; i += blockDim.x)
        if (part[i]) atomicAdd(&cap[i], part[i]);
}

/* the reductions of cuda_get_limit (:820-906) / get_o_limit (:928-1000) over
 * keys [lo, lo + n): offsets with o mod 64 >= 32 do not contribute */
__global__ void __launch_bounds__(1024) k_limits(const u128 *__restrict__ keys, const float4 *__restrict__ boxes,
                                                 const unsigned long long *__restrict__ lo_of,
                                                 const uint32_t *__restrict__ n_of, uint32_t end_time_min,
                                                 uint32_t cur_time, glint_ctf_meta *__restrict__ out) {
    __shared__ float r[4][32];
    __shared__ int rs[2][32];
    const uint32_t c = blockIdx.x;
    const unsigned long long lo = lo_of[c];
    const uint32_t n = n_of[c];
    float l0 = 100000.0f, l1 = 100000.0f, h0 = -100000.0f, h1 = -100000.0f;
    int smin = 1 << 30, smax = 0;
    for (uint32_t o = threadIdx.x; o < n; o += blockDim.x) {
        if ((o & 63u) >= 32u) continue;
        const float4 b = boxes[lo + o];
        l0 = fminf(l0, b.x);
        l1 = fminf(l1, b.y);
        h0 = fmaxf(h0, b.z);
        h1 = fmaxf(h1, b.w);
        const u128 k = keys[lo + o];
        const uint32_t duration = (uint32_t)(k >> 32), end = (uint32_t)k + end_time_min;
        const int st = (int)(end - duration);
        smin = min(smin, st);
        smax = max(smax, st);
    }
    for (int o = 16; o > 0; o >>= 1) {
        l0 = fminf(l0, __shfl_down_sync(0xffffffffu, l0, o));
        l1 = fminf(l1, __shfl_down_sync(0xffffffffu, l1, o));
        h0 = fmaxf(h0, __shfl_down_sync(0xffffffffu, h0, o));
        h1 = fmaxf(h1, __shfl_down_sync(0xffffffffu, h1, o));
        smin = min(smin, __shfl_down_sync(0xffffffffu, smin, o));
        smax = max(smax, __shfl_down_sync(0xffffffffu, smax, o));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        r[0][w] = l0; r[1][w] = l1; r[2][w] = h0; r[3][w] = h1;
        rs[0][w] = smin; rs[1][w] = smax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
            l0 = fminf(l0, r[0][i]); l1 = fminf(l1, r[1][i]);
            h0 = fmaxf(h0, r[2][i]); h1 = fmaxf(h1, r[3][i]);
            smin = min(smin, rs[0][i]); smax = max(smax, rs[1][i]);
        }
        glint_ctf_meta &m = out[c];
        m.ctf_mbr[0] = l0; m.ctf_mbr[1] = l1; m.ctf_mbr[2] = h0; m.ctf_mbr[3] = h1;
        m.CTF_kv_capacity = n;
        m.start_time_min = (uint32_t)smin;
        m.start_time_max = (uint32_t)smax;
        m.end_time_min = end_time_min;
        m.end_time_max = cur_time;
    }
}

__device__ inline void set_bit_global(uint32_t *bits, uint64_t total, uint64_t pos, unsigned long long *outside) {
    if (pos < total) {
        /* many keys set the same bits: bits only go from 0 to 1 here, so a
         * bit already seen set (read at L2) needs no atomic */
        const uint32_t m = 1u << (pos & 31);
        if (!(__ldcg(&bits[pos >> 5]) & m)) atomicOr(&bits[pos >> 5], m);
    } else {
        atomicAdd(outside, 1ull);
    }
}

/* bits x + y * row for x in [l0, h0], y in [l1, h1] from `base`, inside
 * [0, total); a box this large only comes from a box far outside its file's
 * extent: past kBitLoopMax writes the key is reported instead */
constexpr uint64_t kBitLoopMax = 1ull << 22;
__device__ inline void draw_box(uint32_t *bits, uint64_t total, uint64_t base, uint64_t row, uint32_t l0, uint32_t h0,
                                uint32_t l1, uint32_t h1, unsigned long long *outside, DevCounters *cnt) {
    uint64_t n = 0;
    for (uint64_t x = l0; x <= h0 && base + x < total; ++x)
        for (uint64_t y = l1; y <= h1 && base + x + y * row < total; ++y) {
            if (++n > kBitLoopMax) {
                atomicOr(&cnt->error_flags, GLINT_EF_STORE_DOMAIN);
                return;
            }
            set_bit_global(bits, total, base + x + y * row, outside);
        }
}

/* cuda_write_o_bitmap (:908-926): drawn into the bitmap array's first
 * bit_count bits; later bits land in the CTF bitmaps, as the reference's do */
__global__ void k_o_bitmap(const float4 *__restrict__ boxes, uint64_t lo, uint32_t n, double m0, double m1, double m2,
                           double m3, uint32_t *__restrict__ bits, uint64_t total, unsigned long long *outside,
                           DevCounters *cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 b = boxes[lo + i];
        const uint32_t l0 = __double2uint_rz(__dmul_rn(__ddiv_rn(__dsub_rn((double)b.x, m0), __dsub_rn(m2, m0)), 256.0));
        const uint32_t l1 = __double2uint_rz(__dmul_rn(__ddiv_rn(__dsub_rn((double)b.y, m1), __dsub_rn(m3, m1)), 256.0));
        const uint32_t h0 = __double2uint_rz(__dmul_rn(__ddiv_rn(__dsub_rn((double)b.z, m0), __dsub_rn(m2, m0)), 256.0));
        const uint32_t h1 = __double2uint_rz(__dmul_rn(__ddiv_rn(__dsub_rn((double)b.w, m1), __dsub_rn(m3, m1)), 256.0));
        draw_box(bits, total, 0, kBitEdge, l0, h0, l1, h1, outside, cnt);
    }
}

struct CtfTables {
    const glint_ctf_meta *ctfs;
    const unsigned long long *key_index;   /* [C] first key of each CTF */
    const unsigned long long *byte_index;  /* [C] first packed byte of each CTF */
    uint32_t C;
};

/* cuda_write_bitmap (:1003-1034), one thread per key */
__global__ void k_ctf_bitmap(const u128 *__restrict__ keys, const float4 *__restrict__ boxes, uint64_t kv,
                             CtfTables t, uint32_t *__restrict__ bits, uint64_t total,
                             unsigned long long *outside, DevCounters *cnt) {
    for (uint64_t kid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; kid < kv;
         kid += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = key_sid(keys[kid]) - 2u;
        if (c >= t.C) continue;
        const glint_ctf_meta &m = t.ctfs[c];
        const float4 b = boxes[kid];
        const float ex = __fsub_rn(m.ctf_mbr[2], m.ctf_mbr[0]), ey = __fsub_rn(m.ctf_mbr[3], m.ctf_mbr[1]);
        const float xg = (float)m.x_grid, yg = (float)m.y_grid;
        const uint32_t l0 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.x, m.ctf_mbr[0]), ex), xg));
        const uint32_t l1 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.y, m.ctf_mbr[1]), ey), yg));
        const uint32_t h0 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.z, m.ctf_mbr[0]), ex), xg));
        const uint32_t h1 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.w, m.ctf_mbr[1]), ey), yg));
        draw_box(bits, total, (uint64_t)c * kBitCount, m.x_grid, l0, h0, l1, h1, outside, cnt);
    }
}

/* write_key_and_mbr (:1079-1104), one thread per key */
__global__ void k_ctf_pack(const u128 *__restrict__ keys, const float4 *__restrict__ boxes, uint64_t kv, CtfTables t,
                           uint8_t *__restrict__ out, uint64_t out_bytes) {
    for (uint64_t kid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; kid < kv;
         kid += (uint64_t)gridDim.x * blockDim.x) {
        const u128 key = keys[kid];
        const uint32_t c = key_sid(key) - 2u;
        if (c >= t.C) continue;
        const glint_ctf_meta &m = t.ctfs[c];
        const u128 end = key & 0xffffffffu;
        const u128 duration = (key >> 32) & 0xffffffffu;
        const u128 target = (key >> 64) & ((1u << kOidBit) - 1);
        const u128 pid = key >> kPidShift; /* sid included, as extract_fields does */
        const u128 value_mbr = serialize_box(boxes[kid], m);
        const u128 temp = (pid << (m.id_bit + m.duration_bit + m.end_bit + m.mbr_bit)) +
                          (target << (m.duration_bit + m.end_bit + m.mbr_bit)) +
                          (duration << (m.end_bit + m.mbr_bit)) + (end << m.mbr_bit) + value_mbr;
        const uint32_t kb = m.key_bit / 8;
        const uint64_t at = t.byte_index[c] + (kid - t.key_index[c]) * kb;
        if (at + kb > out_bytes) continue;
        put_key_bytes(out + at, temp, kb);
    }
}

/* where each object's keys sit in a flushed block: its CTF part index or its
 * oversize-buffer index, and how many */
/* the earliest meeting start among n unpacked keys (low word: duration << 32
 * | end - base) */
__global__ void k_keys_min_start(const ulonglong2 *__restrict__ keys, uint64_t n, uint32_t base,
                                 uint32_t *__restrict__ out) {
    uint32_t m = 0xffffffffu;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long x = keys[i].x;
        m = min(m, (uint32_t)x + base - (uint32_t)(x >> 32));
    }
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m != 0xffffffffu) atomicMin(out, m);
}

__global__ void k_block_index(uint32_t N, const uint32_t *__restrict__ seg_of, const uint32_t *__restrict__ same,
                              const uint8_t *__restrict__ over, uint64_t kv, uint32_t *__restrict__ first,
                              uint32_t *__restrict__ count) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N; id += gridDim.x * blockDim.x) {
        const uint32_t n = same[id];
        count[id] = n;
        first[id] = n ? (over[id] ? (uint32_t)(seg_of[id] - kv) : seg_of[id]) : 0u;
    }
}

/* CTF::get_ctf_bits + eight_parallel (tracing/step_merge.cpp:132-186) on the
 * host, in the reference's double arithmetic; false where its asserts fire */
uint32_t min_bits_to_store(uint32_t v) {
    if (v == 0) return 1;
    uint32_t b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

bool ctf_bits(glint_ctf_meta &c, const glint_box &map, uint32_t num_objects, uint32_t max_meet_time) {
    c.id_bit = (uint16_t)min_bits_to_store(num_objects);
    c.duration_bit = (uint16_t)min_bits_to_store(max_meet_time - 1);
    c.end_bit = c.duration_bit;
    volatile double map_x_grid_length = (map.high[0] - map.low[0]) / 3000;
    volatile double map_y_grid_length = (map.high[1] - map.low[1]) / 4200;
    volatile double gx = ((double)c.ctf_mbr[2] - (double)c.ctf_mbr[0]) / map_x_grid_length;
    volatile double gy = ((double)c.ctf_mbr[3] - (double)c.ctf_mbr[1]) / map_y_grid_length;
    if (!(gx >= 0.0) || !(gy >= 0.0)) return false;
    const uint32_t low_x_grid = (uint32_t)gx, low_y_grid = (uint32_t)gy;
    c.low_x_bit = (uint16_t)min_bits_to_store(std::max(low_x_grid, 1u) - 1);
    c.low_y_bit = (uint16_t)min_bits_to_store(std::max(low_y_grid, 1u) - 1);
    c.edge_bit = std::max(c.low_x_bit, c.low_y_bit);
    c.mbr_bit = (uint16_t)(c.low_x_bit + c.low_y_bit + 2 * c.edge_bit);
    if (c.mbr_bit > 64) return false;
    const uint32_t temp_bit = c.id_bit * 2u + c.duration_bit + c.end_bit + c.mbr_bit;
    if (temp_bit > 128) return false;
    c.key_bit = (uint16_t)(temp_bit / 8 * 8);
    if (c.key_bit < temp_bit) c.key_bit += 8;
    volatile double wx = ((double)c.ctf_mbr[2] - (double)c.ctf_mbr[0]) / (map.high[0] - map.low[0]) * 300;
    volatile double wy = ((double)c.ctf_mbr[3] - (double)c.ctf_mbr[1]) / (map.high[1] - map.low[1]) * 420;
    const int old_width_grid = (int)wx, old_high_grid = (int)wy;
    int xg = std::max(old_width_grid + 1, 32), yg = std::max(old_high_grid + 1, 32);
    if (xg >= 256 || yg >= 256) {
        xg = std::min(old_width_grid + 1, 255);
        yg = std::min(old_high_grid + 1, 255);
    }
    c.x_grid = (uint16_t)xg;
    c.y_grid = (uint16_t)yg;
    c.ctf_bitmap_size = (uint32_t)(xg * yg + 7) / 8;
    return true;
}

} // namespace glint

using namespace glint;

namespace glint {

cudaError_t flush_alloc(glint_ctx *c) {
    const uint32_t N = c->N;
    const uint64_t cap = c->kv_cap;
    const uint32_t C = c->cfg.CTF_count;
#define FALLOC(p, n)                                                                  \
    do {                                                                              \
        cudaError_t _e = cudaMalloc((void **)&(p), sizeof(*(p)) * ((n) ? (n) : 1));   \
        if (_e != cudaSuccess) return _e;                                             \
    } while (0)
    FALLOC(c->d_keys, cap);
    FALLOC(c->d_keys2, cap);
    FALLOC(c->d_kvbox, cap);
    FALLOC(c->d_kvbox2, cap);
    FALLOC(c->d_same, N);
    FALLOC(c->d_obox, N);
    FALLOC(c->d_sids, N);
    FALLOC(c->d_sids_out, N);
    FALLOC(c->d_over, N);
    FALLOC(c->d_oids, N);
    FALLOC(c->d_oids2, N);
    FALLOC(c->d_mid, N);
    FALLOC(c->d_mid2, N);
    FALLOC(c->d_gcount, (size_t)N + 1);
    FALLOC(c->d_gstart, (size_t)N + 1);
    FALLOC(c->d_segof, N);
    FALLOC(c->d_segcur, N);
    FALLOC(c->d_segbig, N);
    FALLOC(c->d_ctf_cap, C);
    FALLOC(c->d_ctfs, (size_t)C + 1);
    FALLOC(c->d_ctf_lo, (size_t)C + 1);
    FALLOC(c->d_ctf_n, (size_t)C + 1);
    FALLOC(c->d_ctf_byte, C);
    FALLOC(c->d_ctf_keys, cap * 16);
    FALLOC(c->d_bitmaps, (size_t)C * kBitCount / 8);
    FALLOC(c->d_obitmap, kBitCount / 8);
    FALLOC(c->d_fmisc, 8);
    FALLOC(c->d_place, N);
#undef FALLOC
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, radix_tmp_bytes(N));
    if (e != cudaSuccess) return e;
    c->d_rs_tmp = p;
    cudaMemsetAsync(c->d_same, 0, sizeof(uint32_t) * N, c->stream);
    cudaMemsetAsync(c->d_sids, 0, sizeof(uint16_t) * N, c->stream);
    k_init_obox<<<grid_for(N, 256), 256, 0, c->stream>>>(c->d_obox, N);
    return cudaGetLastError();
}

void flush_free(glint_ctx *c) {
    void *ptrs[] = {c->d_keys, c->d_keys2, c->d_kvbox, c->d_kvbox2, c->d_same, c->d_obox, c->d_sids, c->d_sids_out,
                    c->d_over,
                    c->d_oids, c->d_oids2, c->d_mid, c->d_mid2, c->d_gcount, c->d_gstart, c->d_segof, c->d_segcur,
                    c->d_segbig, c->d_ctf_cap, c->d_ctfs, c->d_ctf_lo, c->d_ctf_n, c->d_ctf_byte, c->d_ctf_keys,
                    c->d_bitmaps, c->d_obitmap, c->d_fmisc, c->d_rs_tmp, c->d_place};
    for (void *p : ptrs)
        if (p) cudaFree(p);
}

KeyArgs key_args(glint_ctx *c) {
    KeyArgs a;
    a.keys = reinterpret_cast<u128 *>(c->d_keys);
    a.boxes = c->d_kvbox;
    a.cap = c->kv_cap;
    a.same = c->d_same;
    a.obox = c->d_obox;
    a.sids = c->d_sids;
    a.map[0] = c->mbr.low[0];
    a.map[1] = c->mbr.low[1];
    a.map[2] = c->mbr.high[0];
    a.map[3] = c->mbr.high[1];
    a.max_meet = c->cfg.max_meet_time;
    return a;
}

/* after identify: this step's meetings become keys */
cudaError_t launch_keys(glint_ctx *c) {
    k_keys_append<<<152 * 4, 256, 0, c->stream>>>(c->d_log, c->log_cap, key_args(c), c->d_cnt);
    return cudaGetLastError();
}

void flush_set_attributes() {
    cudaFuncSetAttribute(k_seg_sort_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kSegBlockMax * (sizeof(u128) + sizeof(uint32_t))));
}

/* the whole flush on the context's stream; host synchronisation where the
 * reference's own flush reads counts back */
glint_status run_flush(glint_ctx *c, glint_store_info *info, std::string &err) {
    cudaStream_t s = c->stream;
    const uint32_t N = c->N, C = c->cfg.CTF_count, split = c->cfg.split_num;
    const uint64_t total_bits = (uint64_t)C * kBitCount;
    DevCounters h;
    auto fail = [&](cudaError_t e, const char *where) {
        err = std::string("flush ") + where + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    };
    cudaError_t e;
    /* set_oid and the area cut */
    k_set_oid<<<grid_for(N, 256), 256, 0, s>>>(N, c->d_same, c->d_obox, c->d_sids, c->cfg.dProbFalse, c->d_oids,
                                                c->d_mid, c->d_over, c->d_cnt);
    k_mark_over<<<grid_for(N, 256), 256, 0, s>>>(N, c->d_sids, c->d_over);
    if ((e = cudaMemcpyAsync(&h, c->d_cnt, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(e, "counters");
    const uint64_t old_kv = h.kv_count;
    if (old_kv > c->kv_cap) {
        err = "flush: the key buffer overflowed (kv_capacity)";
        return GLINT_ERR_CAPACITY;
    }
    const uint32_t sid_count = h.sid_count, over_count = h.oversize_oid_count;
    const uint32_t zero_one = (N - sid_count) + over_count;
    const uint32_t M = sid_count - over_count;
    const uint32_t x_part = M / split + 1;
    unsigned long long *d_main = c->d_fmisc;         /* [0] CTF key count */
    unsigned long long *d_outside = c->d_fmisc + 1;  /* [1] bits past the array */
    unsigned int *d_nbig = reinterpret_cast<unsigned int *>(c->d_fmisc + 2);
    cudaMemsetAsync(c->d_fmisc, 0, sizeof(unsigned long long) * 8, s);
    cudaMemsetAsync(c->d_bitmaps, 0, total_bits / 8, s);
    /* d_ctf_keys needs no clearing: the packing writes every byte of the
     * key_bytes it holds, and nothing reads past them */

    /* STR: by mean x (full 64-bit key), then by y inside each x-slice */
    if ((e = radix_sort_u64(c->d_mid, c->d_oids, c->d_mid2, c->d_oids2, N, 64, c->d_rs_tmp, c->d_scan_tmp, s)))
        return fail(e, "STR x sort");
    if (zero_one < N) {
        k_str_slice_keys<<<grid_for(N, 256), 256, 0, s>>>(c->d_mid, N, zero_one, x_part, split);
        int bits = 33;
        while ((1ull << (bits - 32)) <= split) ++bits;
        if ((e = radix_sort_u64(c->d_mid, c->d_oids, c->d_mid2, c->d_oids2, N, bits, c->d_rs_tmp, c->d_scan_tmp, s)))
            return fail(e, "STR y sort");
        k_make_sid<<<grid_for(N, 256), 256, 0, s>>>(c->d_oids, N, zero_one, x_part, split, c->d_sids);
    }

    /* key segments: objects ordered by (oversize part, sid, oid) */
    unsigned long long *gk = c->d_mid;  /* the STR keys are no longer needed */
    uint32_t *gv = c->d_oids2;
    k_group_keys<<<grid_for(N, 256), 256, 0, s>>>(N, c->d_same, c->d_sids, c->d_over, gk, gv);
    if ((e = radix_sort_u64(gk, gv, c->d_mid2, c->d_segbig, N, 42, c->d_rs_tmp, c->d_scan_tmp, s)))
        return fail(e, "object order");
    k_group_counts<<<grid_for(N, 256), 256, 0, s>>>(N, gk, gv, c->d_same, c->d_gcount);
    scan_u32(c->d_gcount, c->d_gstart, N, c->d_scan_tmp, s);
    k_group_starts<<<grid_for(N, 256), 256, 0, s>>>(N, gk, gv, c->d_gstart, c->d_segof, d_main);
    cudaMemsetAsync(c->d_segcur, 0, sizeof(uint32_t) * N, s);
    k_obj_place<<<grid_for(N, 256), 256, 0, s>>>(N, c->d_segof, c->d_sids, c->d_over, c->d_place);
    if (old_kv)
        k_key_scatter<<<grid_for(old_kv, 256, 152u * 16u), 256, 0, s>>>(
            reinterpret_cast<const u128 *>(c->d_keys), c->d_kvbox, old_kv, c->d_place, c->d_segcur,
            reinterpret_cast<u128 *>(c->d_keys2), c->d_kvbox2);
    std::swap(c->d_keys, c->d_keys2);
    std::swap(c->d_kvbox, c->d_kvbox2);
    u128 *keys = reinterpret_cast<u128 *>(c->d_keys);
    /* segments by size: up to 8 keys a thread each, 9..16 two per warp (the
     * per-object cursors of the scatter are free again and list them), up
     * to kSegWarpMax a warp each, longer ones a block each */
    unsigned int *d_nmid = reinterpret_cast<unsigned int *>(c->d_fmisc + 3);
    unsigned int *d_nlarge = reinterpret_cast<unsigned int *>(c->d_fmisc + 4);
    uint32_t *d_large = reinterpret_cast<uint32_t *>(c->d_mid2); /* the group sort's scratch, free again */
    k_seg_sort_tiny<<<grid_for(N, 256), 256, 0, s>>>(gk, gv, c->d_gstart, c->d_same, N, keys, c->d_kvbox,
                                                     c->d_segcur, d_nmid, d_large, d_nlarge);
    k_seg_sort_half<<<152 * 8, 128, 0, s>>>(c->d_segcur, d_nmid, gv, c->d_gstart, c->d_same, keys, c->d_kvbox);
    k_seg_sort_warp<<<152 * 8, 128, 0, s>>>(d_large, d_nlarge, gv, c->d_gstart, c->d_same, keys, c->d_kvbox,
                                           c->d_segbig, d_nbig);
    k_seg_sort_block<<<152, 1024, kSegBlockMax * (sizeof(u128) + sizeof(uint32_t)), s>>>(
        c->d_segbig, gv, c->d_gstart, c->d_same, keys, c->d_kvbox, c->d_kvbox2, c->d_cnt, d_nbig);

    /* CTF capacities, then the part sizes on the host */
    cudaMemsetAsync(c->d_ctf_cap, 0, sizeof(uint32_t) * C, s);
    k_ctf_capacity<<<grid_for(N, 256, 152u * 8u), 256, 0, s>>>(c->d_oids, N, zero_one, c->d_sids, c->d_same, C, c->d_ctf_cap,
                                                    c->d_cnt);
    std::vector<uint32_t> cap(C);
    unsigned long long kv = 0;
    cudaMemcpyAsync(cap.data(), c->d_ctf_cap, sizeof(uint32_t) * C, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&kv, d_main, sizeof(kv), cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e, "capacities");
    if (old_kv == 0 || kv == 0) kv = 0;
    const uint64_t o_n = old_kv - kv;
    uint64_t sum = 0;
    for (uint32_t i = 0; i < C; ++i) sum += cap[i];
    if (sum != kv) {
        err = "flush: CTF capacities do not add up to the key count (meetings longer than max_meet_time)";
        return GLINT_ERR_UNSUPPORTED;
    }

    /* limits of the CTFs and of the oversize buffer (slot C) */
    std::vector<unsigned long long> lo(C + 1), key_index(C), byte_index(C);
    std::vector<uint32_t> nn(C + 1);
    uint64_t acc = 0;
    for (uint32_t i = 0; i < C; ++i) {
        lo[i] = acc;
        key_index[i] = acc;
        nn[i] = cap[i];
        acc += cap[i];
    }
    lo[C] = kv;
    nn[C] = (uint32_t)o_n;
    cudaMemcpyAsync(c->d_ctf_lo, lo.data(), sizeof(unsigned long long) * (C + 1), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_ctf_n, nn.data(), sizeof(uint32_t) * (C + 1), cudaMemcpyHostToDevice, s);
    k_limits<<<C + 1, 1024, 0, s>>>(keys, c->d_kvbox, c->d_ctf_lo, c->d_ctf_n, c->end_time_min, c->last_time,
                                    c->d_ctfs);
    std::vector<glint_ctf_meta> metas(C + 1);
    cudaMemcpyAsync(metas.data(), c->d_ctfs, sizeof(glint_ctf_meta) * (C + 1), cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e, "limits");
    bool ok = true;
    uint64_t bytes = 0;
    for (uint32_t i = 0; i < C; ++i) {
        ok = ctf_bits(metas[i], c->mbr, N, c->cfg.max_meet_time) && ok;
        byte_index[i] = bytes;
        bytes += (uint64_t)cap[i] * metas[i].key_bit / 8;
    }
    if (!ok) {
        err = "flush: a CTF without keys (the reference's get_ctf_bits asserts)";
        return GLINT_ERR_UNSUPPORTED;
    }
    cudaMemcpyAsync(c->d_ctfs, metas.data(), sizeof(glint_ctf_meta) * C, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_ctf_lo, key_index.data(), sizeof(unsigned long long) * C, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_ctf_byte, byte_index.data(), sizeof(unsigned long long) * C, cudaMemcpyHostToDevice, s);

    /* oversize bitmap into the first bitmap's bits, copied out, then cleared */
    uint32_t *bits = reinterpret_cast<uint32_t *>(c->d_bitmaps);
    if (o_n)
        k_o_bitmap<<<grid_for(o_n, 256), 256, 0, s>>>(c->d_kvbox, kv, (uint32_t)o_n, c->mbr.low[0], c->mbr.low[1],
                                                      c->mbr.high[0], c->mbr.high[1], bits, total_bits, d_outside,
                                                      c->d_cnt);
    cudaMemcpyAsync(c->d_obitmap, c->d_bitmaps, kBitCount / 8, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(c->d_bitmaps, 0, kBitCount / 8, s);
    CtfTables t;
    t.ctfs = c->d_ctfs;
    t.key_index = c->d_ctf_lo;
    t.byte_index = c->d_ctf_byte;
    t.C = C;
    if (kv) {
        k_ctf_bitmap<<<grid_for(kv, 256, 152u * 16u), 256, 0, s>>>(keys, c->d_kvbox, kv, t, bits, total_bits,
                                                                    d_outside, c->d_cnt);
        k_ctf_pack<<<grid_for(kv, 256, 152u * 16u), 256, 0, s>>>(keys, c->d_kvbox, kv, t, c->d_ctf_keys,
                                                                  c->kv_cap * 16);
    }
    unsigned long long outside = 0;
    cudaMemcpyAsync(&outside, d_outside, sizeof(outside), cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e, "encode");

    glint_store_info &inf = c->store;
    std::memset(&inf, 0, sizeof(inf));
    inf.kv_count = kv;
    inf.key_bytes = bytes;
    inf.oversize_kv_count = (uint32_t)o_n;
    inf.oversize_start_time_min = metas[C].start_time_min;
    inf.oversize_start_time_max = metas[C].start_time_max;
    inf.oversize_end_time_min = c->end_time_min;
    inf.oversize_end_time_max = c->last_time;
    inf.sid_count = sid_count;
    inf.oversize_oid_count = over_count;
    inf.end_time_min = c->end_time_min;
    inf.cur_time = c->last_time;
    inf.bits_outside = outside;
    c->store_ctf_cap = cap;
    c->store_valid = true;
    if (info) *info = inf;

    /* keep the block on the device for queries */
    if (c->cfg.store_keep) {
        StoreBlock b;
        const size_t bytes_keys = bytes ? bytes : 1;
        cudaError_t ae = cudaSuccess;
        auto A = [&](void **p, size_t n) {
            if (ae == cudaSuccess) ae = cudaMalloc(p, n ? n : 1);
        };
        A((void **)&b.keys, bytes_keys);
        A((void **)&b.ctfs, sizeof(glint_ctf_meta) * C);
        A((void **)&b.key_index, sizeof(unsigned long long) * C);
        A((void **)&b.byte_index, sizeof(unsigned long long) * C);
        A((void **)&b.sids, sizeof(uint16_t) * N);
        A((void **)&b.first, sizeof(uint32_t) * N);
        A((void **)&b.count, sizeof(uint32_t) * N);
        A((void **)&b.okeys, sizeof(ulonglong2) * o_n);
        A((void **)&b.oboxes, sizeof(float4) * o_n);
        A((void **)&b.bitmaps, (size_t)C * kBitCount / 8);
        A((void **)&b.obitmap, kBitCount / 8);
        if (ae != cudaSuccess) {
            store_block_release(b);
            return fail(ae, "keep block");
        }
        if (bytes) cudaMemcpyAsync(b.keys, c->d_ctf_keys, bytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b.ctfs, c->d_ctfs, sizeof(glint_ctf_meta) * C, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b.key_index, c->d_ctf_lo, sizeof(unsigned long long) * C, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b.byte_index, c->d_ctf_byte, sizeof(unsigned long long) * C, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b.sids, c->d_sids, sizeof(uint16_t) * N, cudaMemcpyDeviceToDevice, s);
        if (o_n) {
            cudaMemcpyAsync(b.okeys, c->d_keys + kv, sizeof(ulonglong2) * o_n, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(b.oboxes, c->d_kvbox + kv, sizeof(float4) * o_n, cudaMemcpyDeviceToDevice, s);
        }
        cudaMemcpyAsync(b.bitmaps, c->d_bitmaps, (size_t)C * kBitCount / 8, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(b.obitmap, c->d_obitmap, kBitCount / 8, cudaMemcpyDeviceToDevice, s);
        k_block_index<<<grid_for(N, 256), 256, 0, s>>>(N, c->d_segof, c->d_same, c->d_over, kv, b.first, b.count);
        /* the block's earliest meeting start, for queries that skip blocks
         * outside their time window; the low half of the key count word
         * (cleared right after the keep) holds it meanwhile */
        {
            uint32_t *d_min = reinterpret_cast<uint32_t *>(&c->d_cnt->kv_count);
            cudaMemsetAsync(d_min, 0xff, sizeof(uint32_t), s);
            if (kv + o_n)
                k_keys_min_start<<<grid_for(kv + o_n, 256, 152u * 8u), 256, 0, s>>>(
                    reinterpret_cast<const ulonglong2 *>(c->d_keys), kv + o_n, c->end_time_min, d_min);
            uint32_t m = 0;
            cudaMemcpyAsync(&m, d_min, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            if ((ae = cudaStreamSynchronize(s)) != cudaSuccess) {
                store_block_release(b);
                return fail(ae, "keep block");
            }
            b.start_min = (kv + o_n) ? m : 0;
            b.spans_known = true;
        }
        b.kv = kv;
        b.o_count = o_n;
        b.key_bytes = bytes;
        b.end_time_min = c->end_time_min;
        b.end_time_max = c->last_time;
        b.C = C;
        b.o_times[0] = inf.oversize_start_time_min;
        b.o_times[1] = inf.oversize_start_time_max;
        b.o_times[2] = inf.oversize_end_time_min;
        b.o_times[3] = inf.oversize_end_time_max;
        b.sid_count = inf.sid_count;
        b.oversize_oid_count = inf.oversize_oid_count;
        c->ctbs.push_back(b);
        if ((ae = store_blocks_trim(c)) != cudaSuccess) return fail(ae, "keep block in host memory");
    }

    /* the next window (cuda/geometry.cu:2112-2131, tracing/process.cpp:271,549);
     * the sids array is kept as the store's and cleared at the next key */
    cudaMemcpyAsync(c->d_sids_out, c->d_sids, sizeof(uint16_t) * N, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(c->d_sids, 0, sizeof(uint16_t) * N, s);
    cudaMemsetAsync(c->d_same, 0, sizeof(uint32_t) * N, s);
    k_init_obox<<<grid_for(N, 256), 256, 0, s>>>(c->d_obox, N);
    cudaMemsetAsync(&c->d_cnt->kv_count, 0, sizeof(unsigned long long) + 3 * sizeof(unsigned int), s);
    /* the sorted buffers hold the store; new keys go to the other pair */
    c->store_keys_ptr = c->d_keys;
    c->store_boxes_ptr = c->d_kvbox;
    c->store_kv = kv;
    std::swap(c->d_keys, c->d_keys2);
    std::swap(c->d_kvbox, c->d_kvbox2);
    c->end_time_min = c->last_time;
    c->flushes++;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e, "reset");
    return GLINT_OK;
}

} // namespace glint

/* glint_serve_only: the meeting table, the meeting log and the pending-key
 * buffers are released; host-kept blocks move back to the device, oldest
 * first, while more than `reserve` bytes stay free */
extern "C" glint_status glint_serve_only(glint_ctx *c, uint64_t reserve, uint32_t *blocks_on_device) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        c->last_error = std::string("serve only: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    if (!c->serve_only) {
        void **big[] = {(void **)&c->d_tab, (void **)&c->d_stamp, (void **)&c->d_newline, (void **)&c->d_new,
                        (void **)&c->d_log, (void **)&c->d_keys, (void **)&c->d_keys2, (void **)&c->d_kvbox,
                        (void **)&c->d_kvbox2, (void **)&c->d_ctf_keys};
        for (void **p : big) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        c->serve_only = true;
        c->store_valid = false;
        c->stats_valid = false;
    }
    const size_t N = c->N;
    for (StoreBlock &b : c->ctbs) {
        if (!b.on_host) continue;
        void **fields[] = {(void **)&b.keys, (void **)&b.ctfs, (void **)&b.key_index, (void **)&b.byte_index,
                           (void **)&b.sids, (void **)&b.first, (void **)&b.count, (void **)&b.okeys,
                           (void **)&b.oboxes, (void **)&b.bitmaps, (void **)&b.obitmap};
        const size_t bytes[] = {b.key_bytes ? b.key_bytes : 1, sizeof(glint_ctf_meta) * b.C,
                                sizeof(unsigned long long) * b.C, sizeof(unsigned long long) * b.C,
                                sizeof(uint16_t) * N, sizeof(uint32_t) * N, sizeof(uint32_t) * N,
                                sizeof(ulonglong2) * b.o_count, sizeof(float4) * b.o_count,
                                (size_t)b.C * kBitCount / 8, kBitCount / 8};
        constexpr int F = sizeof(bytes) / sizeof(bytes[0]);
        size_t total = 0, free_b = 0, all_b = 0;
        for (size_t x : bytes) total += x;
        if (cudaMemGetInfo(&free_b, &all_b) != cudaSuccess || free_b < total + reserve) break;
        void *dev[F] = {};
        e = cudaSuccess;
        for (int i = 0; i < F && e == cudaSuccess; ++i) e = cudaMalloc(&dev[i], bytes[i] ? bytes[i] : 1);
        for (int i = 0; i < F && e == cudaSuccess; ++i)
            if (bytes[i] && *fields[i]) e = cudaMemcpyAsync(dev[i], *fields[i], bytes[i], cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            for (int i = 0; i < F; ++i)
                if (dev[i]) cudaFree(dev[i]);
            cudaGetLastError();
            break;
        }
        for (int i = 0; i < F; ++i) {
            if (*fields[i]) cudaFreeHost(*fields[i]);
            *fields[i] = dev[i];
        }
        b.on_host = false;
    }
    if (blocks_on_device) {
        uint32_t n = 0;
        for (const StoreBlock &b : c->ctbs) n += b.on_host ? 0u : 1u;
        *blocks_on_device = n;
    }
    return GLINT_OK;
}

extern "C" glint_status glint_flush(glint_ctx *c, glint_store_info *info) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "flush")) return GLINT_ERR_STATE;
    if (c->step_index == 0) {
        c->last_error = "flush before the first step";
        return GLINT_ERR_STATE;
    }
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        c->last_error = std::string("flush: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    std::string err;
    const glint_status st = run_flush(c, info, err);
    if (st != GLINT_OK) c->last_error = err;
    return st;
}

extern "C" glint_status glint_store_read(glint_ctx *c, uint8_t *keys, uint16_t *sids, uint32_t *ctf_capacity,
                                         glint_ctf_meta *ctfs, uint8_t *bitmaps, void *oversize_keys,
                                         float *oversize_boxes, uint8_t *oversize_bitmap, glint_store_info *info) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    if (!c->store_valid) {
        c->last_error = "no flush yet";
        return GLINT_ERR_STATE;
    }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    const glint_store_info &inf = c->store;
    const uint32_t C = c->cfg.CTF_count;
    cudaError_t e = cudaSuccess;
    if (keys && inf.key_bytes) e = cudaMemcpy(keys, c->d_ctf_keys, inf.key_bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && sids)
        e = cudaMemcpy(sids, c->d_sids_out, sizeof(uint16_t) * c->N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && ctf_capacity) std::memcpy(ctf_capacity, c->store_ctf_cap.data(), sizeof(uint32_t) * C);
    if (e == cudaSuccess && ctfs) e = cudaMemcpy(ctfs, c->d_ctfs, sizeof(glint_ctf_meta) * C, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && bitmaps)
        e = cudaMemcpy(bitmaps, c->d_bitmaps, (size_t)C * kBitCount / 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && oversize_keys && inf.oversize_kv_count)
        e = cudaMemcpy(oversize_keys, reinterpret_cast<const u128 *>(c->store_keys_ptr) + c->store_kv,
                       sizeof(u128) * inf.oversize_kv_count, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && oversize_boxes && inf.oversize_kv_count)
        e = cudaMemcpy(oversize_boxes, c->store_boxes_ptr + c->store_kv, sizeof(float4) * inf.oversize_kv_count,
                       cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && oversize_bitmap)
        e = cudaMemcpy(oversize_bitmap, c->d_obitmap, kBitCount / 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        c->last_error = std::string("store read: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    if (info) *info = inf;
    return GLINT_OK;
}

namespace glint {
void store_block_release(StoreBlock &b) {
    void *ps[] = {b.keys,  b.ctfs,  b.key_index, b.byte_index, b.sids,   b.first,
                  b.count, b.okeys, b.oboxes,    b.bitmaps,    b.obitmap};
    for (void *p : ps)
        if (p) {
            if (b.on_host) cudaFreeHost(p);
            else cudaFree(p);
        }
    b = StoreBlock();
}

/* a device-kept block's arrays into page-locked host memory.  On this
 * platform a page-locked allocation is addressed by the GPU at its host
 * address (unified addressing), so the block's pointers stay valid for the
 * query kernels; where the device address differs, or host memory runs
 * out, the block is not moved (moved = false). */
static cudaError_t block_to_host(glint_ctx *c, StoreBlock &b, bool &moved) {
    moved = false;
    const size_t N = c->N;
    void **fields[] = {(void **)&b.keys, (void **)&b.ctfs, (void **)&b.key_index, (void **)&b.byte_index,
                       (void **)&b.sids, (void **)&b.first, (void **)&b.count, (void **)&b.okeys,
                       (void **)&b.oboxes, (void **)&b.bitmaps, (void **)&b.obitmap};
    const size_t bytes[] = {b.key_bytes ? b.key_bytes : 1, sizeof(glint_ctf_meta) * b.C,
                            sizeof(unsigned long long) * b.C, sizeof(unsigned long long) * b.C,
                            sizeof(uint16_t) * N, sizeof(uint32_t) * N, sizeof(uint32_t) * N,
                            sizeof(ulonglong2) * b.o_count, sizeof(float4) * b.o_count,
                            (size_t)b.C * kBitCount / 8, kBitCount / 8};
    constexpr int F = sizeof(bytes) / sizeof(bytes[0]);
    void *host[F] = {};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < F && e == cudaSuccess; ++i) {
        e = cudaHostAlloc(&host[i], bytes[i] ? bytes[i] : 1, cudaHostAllocMapped);
        void *dp = nullptr;
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&dp, host[i], 0);
        if (e == cudaSuccess && dp != host[i]) e = cudaErrorNotSupported;
    }
    for (int i = 0; i < F && e == cudaSuccess; ++i)
        if (bytes[i] && *fields[i]) e = cudaMemcpyAsync(host[i], *fields[i], bytes[i], cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        for (int i = 0; i < F; ++i)
            if (host[i]) cudaFreeHost(host[i]);
        if (e == cudaErrorNotSupported || e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            return cudaSuccess;
        }
        return e;
    }
    for (int i = 0; i < F; ++i) {
        if (*fields[i]) cudaFree(*fields[i]);
        *fields[i] = host[i];
    }
    b.on_host = true;
    moved = true;
    return cudaSuccess;
}

bool serve_only_refused(glint_ctx *c, const char *what) {
    if (!c->serve_only) return false;
    c->last_error = std::string(what) + ": the context serves queries only (glint_serve_only)";
    return true;
}

cudaError_t store_blocks_trim(glint_ctx *c) {
    /* kept blocks run oldest to newest */
    for (;;) {
        size_t host = 0, dev = 0, oldest_dev = c->ctbs.size();
        for (size_t i = 0; i < c->ctbs.size(); ++i) {
            if (c->ctbs[i].on_host) {
                ++host;
            } else {
                if (oldest_dev == c->ctbs.size()) oldest_dev = i;
                ++dev;
            }
        }
        if (host > c->cfg.store_host_keep) {
            /* the oldest host-kept block goes */
            for (size_t i = 0; i < c->ctbs.size(); ++i)
                if (c->ctbs[i].on_host) {
                    store_block_release(c->ctbs[i]);
                    c->ctbs.erase(c->ctbs.begin() + (long)i);
                    break;
                }
            continue;
        }
        if (dev <= c->cfg.store_keep) break;
        cudaStreamSynchronize(c->stream);
        bool moved = false;
        if (c->cfg.store_host_keep) {
            cudaError_t e = block_to_host(c, c->ctbs[oldest_dev], moved);
            if (e != cudaSuccess) return e;
        }
        if (!moved) {
            /* no host tier, or no room for it there: the oldest device block goes */
            store_block_release(c->ctbs[oldest_dev]);
            c->ctbs.erase(c->ctbs.begin() + (long)oldest_dev);
        }
    }
    return cudaSuccess;
}

void store_blocks_free(glint_ctx *c) {
    for (StoreBlock &o : c->ctbs) store_block_release(o);
    c->ctbs.clear();
}
} // namespace glint
