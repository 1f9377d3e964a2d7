/*
 * k_sort.cu -- stable LSD radix sort of (u64 key, u32 value) pairs, used by
 * the flush (object orders and the STR partition).
 *
 * The reference sorts with thrust::sort_by_key, a stable radix sort for
 * primitive keys (cuda/geometry.cu:1865,1881-1890); ties must keep their
 * input order, so every pass here is stable.
 *
 * One pass over 8 key bits, in tiles of 2048 consecutive elements.  Pass 1
 * counts the digits of every tile (shared-memory histograms); an exclusive
 * scan over the digit-major table gives each (digit, tile) its output base;
 * pass 2 ranks every key among the tile's keys of its digit (each warp walks
 * its 256 keys in order, equal digits in a 32-key chunk ranked with
 * __match_any_sync), gathers the tile digit by digit in shared memory and
 * writes each digit's run with consecutive threads on consecutive output
 * elements, so the writes coalesce.  Equal keys leave in input order.
 * Passes only cover the key bits that can be non-zero (the caller gives the
 * bit count).
 */
#include "glint_internal.cuh"

namespace glint {

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsItems = 8;                              /* keys per thread */
constexpr uint32_t kRsTile = kRsThreads * kRsItems;      /* 2048 keys per tile */
constexpr int kRsDigits = 256;

/* digit counts of every tile, digit-major: cnt[d * tiles + t] */
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const unsigned long long *__restrict__ keys, uint64_t n,
                                                        int shift, uint32_t *__restrict__ cnt, uint64_t tiles) {
    __shared__ uint32_t h[kRsDigits];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t t = blockIdx.x;
    const uint64_t b = t * kRsTile;
    const uint64_t e = b + kRsTile < n ? b + kRsTile : n;
    for (uint64_t i = b + threadIdx.x; i < e; i += kRsThreads) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1u);
    __syncthreads();
    cnt[(uint64_t)threadIdx.x * tiles + t] = h[threadIdx.x];
}

/* one tile: ranks every key among the tile's keys of its digit (stable: warp
 * w holds keys [256 w, 256 w + 256) of the tile, in chunks of 32), gathers the
 * tile digit by digit in shared memory, then writes each digit's run to its
 * place in the output with consecutive threads on consecutive elements */
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const unsigned long long *__restrict__ keys,
                                                           const uint32_t *__restrict__ vals, uint64_t n, int shift,
                                                           const uint32_t *__restrict__ off, uint64_t tiles,
                                                           unsigned long long *__restrict__ okeys,
                                                           uint32_t *__restrict__ ovals) {
    __shared__ unsigned long long sk[kRsTile];
    __shared__ uint32_t sv[kRsTile];
    __shared__ uint32_t wcnt[kRsWarps][kRsDigits];
    __shared__ uint32_t dstart[kRsDigits];
    __shared__ uint32_t gbase[kRsDigits];
    __shared__ uint32_t wsum[kRsWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t t = blockIdx.x;
    const uint64_t b = t * kRsTile;
    const uint64_t e = b + kRsTile < n ? b + kRsTile : n;
    for (int d = lane; d < kRsDigits; d += 32) wcnt[w][d] = 0;
    __syncwarp();
    unsigned long long k[kRsItems];
    uint32_t v[kRsItems], dg[kRsItems], rank[kRsItems];
#pragma unroll
    for (int c = 0; c < kRsItems; ++c) {
        const uint64_t i = b + (uint64_t)w * (32 * kRsItems) + c * 32 + lane;
        const bool valid = i < e;
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        k[c] = valid ? keys[i] : 0ull;
        v[c] = valid ? vals[i] : 0u;
        dg[c] = (uint32_t)((k[c] >> shift) & 0xff);
        uint32_t lt = 0, peers = 0, base = 0;
        if (valid) {
            peers = __match_any_sync(active, dg[c]);
            lt = __popc(peers & ((1u << lane) - 1u));
            base = wcnt[w][dg[c]];
        }
        rank[c] = valid ? base + lt : 0xffffffffu;
        __syncwarp();
        if (valid && lt == 0) wcnt[w][dg[c]] = base + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    /* per digit: warps' offsets, then the tile's digit starts */
    const int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < kRsWarps; ++ww) {
        const uint32_t x = wcnt[ww][d];
        wcnt[ww][d] = run;
        run += x;
    }
    uint32_t x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    gbase[d] = off[(uint64_t)d * tiles + t];
    __syncthreads();
    uint32_t before = 0;
    for (int ww = 0; ww < w; ++ww) before += wsum[ww];
    dstart[d] = before + x - run;
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kRsItems; ++c)
        if (rank[c] != 0xffffffffu) {
            const uint32_t pos = dstart[dg[c]] + wcnt[w][dg[c]] + rank[c];
            sk[pos] = k[c];
            sv[pos] = v[c];
        }
    __syncthreads();
    const uint32_t cnt = (uint32_t)(e - b);
    for (uint32_t q = threadIdx.x; q < cnt; q += kRsThreads) {
        const unsigned long long kk = sk[q];
        const uint32_t dd = (uint32_t)((kk >> shift) & 0xff);
        const uint64_t g = (uint64_t)gbase[dd] + (q - dstart[dd]);
        okeys[g] = kk;
        ovals[g] = sv[q];
    }
}

size_t radix_tmp_bytes(uint64_t n) {
    const uint64_t tiles = (n + kRsTile - 1) / kRsTile;
    /* the digit tables, then the keys' OR and AND (radix_sort_u64_varying) */
    return sizeof(uint32_t) * ((size_t)kRsDigits * (tiles ? tiles : 1) + 1) * 2 + 2 * sizeof(unsigned long long);
}

/* OR and AND of all keys: the bits that vary */
__global__ void __launch_bounds__(256) k_rs_bits(const unsigned long long *__restrict__ keys, uint64_t n,
                                                 unsigned long long *__restrict__ orand) {
    unsigned long long o = 0, a = ~0ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        o |= k;
        a &= k;
    }
    for (int d = 16; d > 0; d >>= 1) {
        o |= __shfl_xor_sync(0xffffffffu, o, d);
        a &= __shfl_xor_sync(0xffffffffu, a, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicOr(&orand[0], o);
        atomicAnd(&orand[1], a);
    }
}

/* Sorts (keys, vals)[0, n) stably by the low `bits` bits of the keys.  tmp_k /
 * tmp_v hold n elements; rs_tmp holds radix_tmp_bytes(n); scan_tmp is scan
 * scratch for 256 * ceil(n / 1024) + 1 values.  The result is left in keys /
 * vals. */
cudaError_t radix_sort_u64(unsigned long long *keys, uint32_t *vals, unsigned long long *tmp_k, uint32_t *tmp_v,
                           uint64_t n, int bits, void *rs_tmp, void *scan_tmp, cudaStream_t s) {
    if (n < 2 || bits <= 0) return cudaSuccess;
    const uint64_t tiles = (n + kRsTile - 1) / kRsTile;
    if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
    uint32_t *cnt = static_cast<uint32_t *>(rs_tmp);
    uint32_t *off = cnt + (size_t)kRsDigits * tiles + 1;
    unsigned long long *src_k = keys, *dst_k = tmp_k;
    uint32_t *src_v = vals, *dst_v = tmp_v;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8, ++passes) {
        k_rs_hist<<<(unsigned)tiles, kRsThreads, 0, s>>>(src_k, n, shift, cnt, tiles);
        cudaError_t e = scan_u32(cnt, off, (size_t)kRsDigits * tiles, scan_tmp, s);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<(unsigned)tiles, kRsThreads, 0, s>>>(src_k, src_v, n, shift, off, tiles, dst_k, dst_v);
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, src_k, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, src_v, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
    }
    return cudaGetLastError();
}

/* The same sort, without the passes whose 8-bit digit is equal in every key
 * (such a pass moves nothing): one reduction of the keys' OR and AND, read on
 * the host, picks the passes.  Synchronises the stream once. */
cudaError_t radix_sort_u64_varying(unsigned long long *keys, uint32_t *vals, unsigned long long *tmp_k,
                                   uint32_t *tmp_v, uint64_t n, int bits, void *rs_tmp, void *scan_tmp,
                                   cudaStream_t s) {
    if (n < 2 || bits <= 0) return cudaSuccess;
    const uint64_t tiles = (n + kRsTile - 1) / kRsTile;
    if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
    uint32_t *cnt = static_cast<uint32_t *>(rs_tmp);
    uint32_t *off = cnt + (size_t)kRsDigits * tiles + 1;
    unsigned long long *orand =
        reinterpret_cast<unsigned long long *>(static_cast<uint8_t *>(rs_tmp) + radix_tmp_bytes(n) - 16);
    cudaMemsetAsync(orand, 0, sizeof(unsigned long long), s);
    cudaMemsetAsync(orand + 1, 0xff, sizeof(unsigned long long), s);
    k_rs_bits<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 152 * 8), 256, 0, s>>>(keys, n, orand);
    unsigned long long h[2];
    cudaError_t e = cudaMemcpyAsync(h, orand, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    const unsigned long long varying = h[0] ^ h[1];
    unsigned long long *src_k = keys, *dst_k = tmp_k;
    uint32_t *src_v = vals, *dst_v = tmp_v;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        if (!((varying >> shift) & 0xffull)) continue;
        k_rs_hist<<<(unsigned)tiles, kRsThreads, 0, s>>>(src_k, n, shift, cnt, tiles);
        e = scan_u32(cnt, off, (size_t)kRsDigits * tiles, scan_tmp, s);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<(unsigned)tiles, kRsThreads, 0, s>>>(src_k, src_v, n, shift, off, tiles, dst_k, dst_v);
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
        ++passes;
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
