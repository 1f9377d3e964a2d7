/*
 * store_codec.cuh -- the store's box quantisation, shared by the flush and
 * the compaction of kept blocks.
 */
#ifndef GLINT_STORE_CODEC_CUH_
#define GLINT_STORE_CODEC_CUH_

#include <cstdint>

#include "glint.h"

namespace glint {

/* serialize_mbr for f_box (cuda/geometry.cu:162-174): float arithmetic,
 * truncated to integers */
__device__ inline uint64_t serialize_box(const float4 &b, const glint_ctf_meta &m) {
    const float ex = __fsub_rn(m.ctf_mbr[2], m.ctf_mbr[0]), ey = __fsub_rn(m.ctf_mbr[3], m.ctf_mbr[1]);
    const float longer_edge = fmaxf(ex, ey);
    const float fx = __ull2float_rn((1ull << m.low_x_bit) - 1), fy = __ull2float_rn((1ull << m.low_y_bit) - 1);
    const float fe = __ull2float_rn((1ull << m.edge_bit) - 1);
    const uint64_t low0 = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.x, m.ctf_mbr[0]), ex), fx));
    const uint64_t low1 = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.y, m.ctf_mbr[1]), ey), fy));
    const uint64_t x = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.z, b.x), longer_edge), fe));
    const uint64_t y = __float2ull_rz(__fmul_rn(__fdiv_rn(__fsub_rn(b.w, b.y), longer_edge), fe));
    return (low0 << (m.low_y_bit + m.edge_bit + m.edge_bit)) + (low1 << (m.edge_bit + m.edge_bit)) +
           (x << m.edge_bit) + y;
}

/* a packed key's kb little-endian bytes (kb <= 16).  The loops are unrolled
 * over the 16 possible bytes, so every shift is a constant on a 64-bit half;
 * a loop over kb with a 128-bit shift by 8 j costs a long shift sequence per
 * byte. */
__device__ inline void put_key_bytes(uint8_t *dst, unsigned __int128 key, uint32_t kb) {
    const uint64_t lo = (uint64_t)key, hi = (uint64_t)(key >> 64);
#pragma unroll
    for (int j = 0; j < 16; ++j)
        if ((uint32_t)j < kb) dst[j] = (uint8_t)(j < 8 ? lo >> (8 * j) : hi >> (8 * (j - 8)));
}

__device__ inline unsigned __int128 get_key_bytes(const uint8_t *src, uint32_t kb) {
    uint64_t lo = 0, hi = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j)
        if ((uint32_t)j < kb) {
            const uint64_t b = src[j];
            if (j < 8) lo |= b << (8 * j);
            else hi |= b << (8 * (j - 8));
        }
    return ((unsigned __int128)hi << 64) | lo;
}

/* kb <= 16 little-endian bytes at p, read as whole 8-byte words where
 * they stay inside the buffer ending at `end` (whose start is 8-aligned),
 * else byte by byte */
__device__ inline unsigned __int128 load_key(const uint8_t *p, uint32_t kb, const uint8_t *end) {
    const uintptr_t a = (uintptr_t)p;
    const uint64_t *w = (const uint64_t *)(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7) * 8;
    unsigned __int128 v;
    if ((const uint8_t *)(w + 3) <= end) {
        const uint64_t w0 = w[0], w1 = w[1];
        v = ((unsigned __int128)w1 << 64 | w0) >> sh;
        if (sh) v |= (unsigned __int128)w[2] << (128 - sh);
    } else {
        return get_key_bytes(p, kb);
    }
    return kb < 16 ? v & (((unsigned __int128)1 << (8 * kb)) - 1) : v;
}

} // namespace glint

#endif
