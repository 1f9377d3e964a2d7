/*
 * k_sort.cu -- stable LSD radix sort of (u64 key, u32 value) pairs, used by
 * the flush (object orders and the STR partition).
 *
 * The reference sorts with thrust::sort_by_key, a stable radix sort for
 * primitive keys (cuda/geometry.cu:1865,1881-1890); ties must keep their
 * input order, so every pass here is stable.
 *
 * One pass over 8 key bits: each warp owns a range of 1024 consecutive
 * elements.  Pass 1 counts the digits of every warp range (shared-memory
 * histograms); an exclusive scan over the digit-major table gives each
 * (digit, range) its output base; pass 2 walks each range in element order
 * and ranks equal digits inside a 32-element chunk with __match_any_sync, so
 * equal keys leave in input order.  Passes only cover the key bits that can
 * be non-zero (the caller gives the bit count).
 */
#include "glint_internal.cuh"

namespace glint {

constexpr int kRsWarps = 8;
constexpr uint32_t kRsRange = 1024; /* elements per warp range */
constexpr int kRsDigits = 256;

__global__ void __launch_bounds__(32 * kRsWarps) k_rs_hist(const unsigned long long *__restrict__ keys, uint64_t n,
                                                           int shift, uint32_t *__restrict__ cnt, uint64_t ranges) {
    __shared__ uint32_t h[kRsWarps][kRsDigits];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t r = (uint64_t)blockIdx.x * kRsWarps + w;
    for (int d = lane; d < kRsDigits; d += 32) h[w][d] = 0;
    __syncwarp();
    if (r < ranges) {
        const uint64_t b = r * kRsRange;
        const uint64_t e = b + kRsRange < n ? b + kRsRange : n;
        for (uint64_t i = b + lane; i < e; i += 32) atomicAdd(&h[w][(keys[i] >> shift) & 0xff], 1u);
        __syncwarp();
        for (int d = lane; d < kRsDigits; d += 32) cnt[(uint64_t)d * ranges + r] = h[w][d];
    }
}

__global__ void __launch_bounds__(32 * kRsWarps) k_rs_scatter(const unsigned long long *__restrict__ keys,
                                                              const uint32_t *__restrict__ vals, uint64_t n, int shift,
                                                              const uint32_t *__restrict__ off, uint64_t ranges,
                                                              unsigned long long *__restrict__ okeys,
                                                              uint32_t *__restrict__ ovals) {
    __shared__ uint32_t base[kRsWarps][kRsDigits];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t r = (uint64_t)blockIdx.x * kRsWarps + w;
    if (r >= ranges) return;
    for (int d = lane; d < kRsDigits; d += 32) base[w][d] = off[(uint64_t)d * ranges + r];
    __syncwarp();
    const uint64_t b = r * kRsRange;
    const uint64_t e = b + kRsRange < n ? b + kRsRange : n;
    for (uint64_t c = b; c < e; c += 32) {
        const uint64_t i = c + lane;
        const bool valid = i < e;
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        unsigned long long k = 0;
        uint32_t v = 0, d = 0;
        if (valid) {
            k = keys[i];
            v = vals[i];
            d = (uint32_t)((k >> shift) & 0xff);
        }
        if (valid) {
            const unsigned peers = __match_any_sync(active, d);
            const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
            const uint32_t pos = base[w][d] + rank;
            okeys[pos] = k;
            ovals[pos] = v;
            __syncwarp(active);
            if (rank == 0) base[w][d] += __popc(peers);
        }
        __syncwarp();
    }
}

size_t radix_tmp_bytes(uint64_t n) {
    const uint64_t ranges = (n + kRsRange - 1) / kRsRange;
    return sizeof(uint32_t) * ((size_t)kRsDigits * (ranges ? ranges : 1) + 1) * 2;
}

/* Sorts (keys, vals)[0, n) stably by the low `bits` bits of the keys.  tmp_k /
 * tmp_v hold n elements; rs_tmp holds radix_tmp_bytes(n); scan_tmp is the
 * context's scan scratch (sized for 256 * ranges + 1).  The result is left in
 * keys / vals. */
cudaError_t radix_sort_u64(unsigned long long *keys, uint32_t *vals, unsigned long long *tmp_k, uint32_t *tmp_v,
                           uint64_t n, int bits, void *rs_tmp, void *scan_tmp, cudaStream_t s) {
    if (n < 2 || bits <= 0) return cudaSuccess;
    const uint64_t ranges = (n + kRsRange - 1) / kRsRange;
    uint32_t *cnt = static_cast<uint32_t *>(rs_tmp);
    uint32_t *off = cnt + (size_t)kRsDigits * ranges + 1;
    const unsigned blocks = (unsigned)((ranges + kRsWarps - 1) / kRsWarps);
    unsigned long long *src_k = keys, *dst_k = tmp_k;
    uint32_t *src_v = vals, *dst_v = tmp_v;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8, ++passes) {
        k_rs_hist<<<blocks, 32 * kRsWarps, 0, s>>>(src_k, n, shift, cnt, ranges);
        cudaError_t e = scan_u32(cnt, off, (size_t)kRsDigits * ranges, scan_tmp, s);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<blocks, 32 * kRsWarps, 0, s>>>(src_k, src_v, n, shift, off, ranges, dst_k, dst_v);
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, src_k, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, src_v, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
    }
    return cudaGetLastError();
}

/* number of radix passes' worth of bits needed for keys below 2^bits */
int radix_bits_for(unsigned long long max_key) {
    int b = 0;
    while (b < 64 && (max_key >> b)) ++b;
    return b;
}

} // namespace glint
