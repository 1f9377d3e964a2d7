/*
 * k_util.cu -- device-wide exclusive scan, the double-double sin
 * coefficients, and the device side of the synthetic trajectory generator.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "glint_internal.cuh"
#include "tracegen.h"

namespace glint {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

size_t scan_tmp_bytes(size_t n) {
    size_t tiles = (n + kScanTile - 1) / kScanTile + 1;
    return (tiles + 1) * sizeof(uint32_t);
}

__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums, uint32_t &block_total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t prefix = (wid > 0 ? warp_sums[wid - 1] : 0u) + x - v;
    block_total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return prefix;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t *in, size_t n, uint32_t *tile_sums) {
    __shared__ uint32_t ws[32];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_exclusive_scan(s, ws, tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

/* one block: exclusive scan of the tile sums in place; total into tile_sums[tiles] */
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(uint32_t *tile_sums, size_t tiles) {
    __shared__ uint32_t ws[32];
    uint32_t carry = 0;
    for (size_t base = 0; base < tiles; base += kScanThreads) {
        size_t i = base + threadIdx.x;
        uint32_t v = i < tiles ? tile_sums[i] : 0u;
        uint32_t tot;
        uint32_t p = block_exclusive_scan(v, ws, tot);
        if (i < tiles) tile_sums[i] = carry + p;
        carry += tot;
    }
    if (threadIdx.x == 0) tile_sums[tiles] = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const uint32_t *in, uint32_t *out, size_t n,
                                                           const uint32_t *tile_off, size_t tiles) {
    __shared__ uint32_t ws[32];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t tot;
    uint32_t p = block_exclusive_scan(s, ws, tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = p;
        p += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = tile_off[tiles];
}

cudaError_t scan_u32(const uint32_t *in, uint32_t *out, size_t n, void *tmp, cudaStream_t s) {
    size_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) tiles = 1;
    uint32_t *ts = (uint32_t *)tmp;
    k_scan_reduce<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, ts);
    k_scan_tiles<<<1, kScanThreads, 0, s>>>(ts, tiles);
    k_scan_down<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, ts, tiles);
    return cudaGetLastError();
}

/* ---- double-double Taylor coefficients (-1)^k/(2k+1)!, computed on the host
 * in double-double with the same two-product/two-sum steps ---- */
static inline void h_quick(double a, double b, double &s, double &e) {
    s = a + b;
    e = b - (s - a);
}
static inline void h_div(double ah, double al, double d, double &qh, double &ql) {
    double q1 = ah / d;
    double p = q1 * d;
    double pe = std::fma(q1, d, -p);
    double r = ((ah - p) - pe) + al;
    double q2 = r / d;
    h_quick(q1, q2, qh, ql);
}

void init_sin_coef(SinCoef *c) {
    double fh = 1.0, fl = 0.0;
    c->hi[0] = 1.0;
    c->lo[0] = 0.0;
    for (int k = 1; k <= 20; ++k) {
        h_div(fh, fl, (double)(2 * k), fh, fl);
        h_div(fh, fl, (double)(2 * k + 1), fh, fl);
        c->hi[k] = (k & 1) ? -fh : fh;
        c->lo[k] = (k & 1) ? -fl : fl;
    }
}

} // namespace glint

/* ---- device trajectory generator ---- */
struct glint_gen {
    tg_params *d_params = nullptr;
    tg_object *d_objects = nullptr;
    uint32_t n = 0;
    uint32_t step = 0;    /* index of the next step produced */
};

__global__ void k_gen_step(const tg_params *__restrict__ P, tg_object *__restrict__ objs, uint32_t n, uint32_t step,
                           double *__restrict__ out) {
    const tg_params p = *P;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        tg_object o = objs[i];
        if (step > 0) tg_advance(&p, &o, i, step);
        double lon, lat;
        tg_position(&p, &o, &lon, &lat);
        objs[i] = o;
        reinterpret_cast<double2 *>(out)[i] = make_double2(lon, lat);
    }
}

extern "C" {

glint_status glint_gen_create(const void *params, uint32_t params_size, const void *objects, uint32_t num_objects,
                              uint32_t object_size, uint32_t first_step, glint_gen **out) {
    if (!params || !objects || !out || params_size != sizeof(tg_params) || object_size != sizeof(tg_object))
        return GLINT_ERR_INVALID_ARGUMENT;
    glint_gen *g = new glint_gen();
    g->n = num_objects;
    g->step = first_step;
    if (cudaMalloc(&g->d_params, sizeof(tg_params)) != cudaSuccess ||
        cudaMalloc(&g->d_objects, sizeof(tg_object) * (size_t)(num_objects ? num_objects : 1)) != cudaSuccess) {
        cudaFree(g->d_params);
        delete g;
        return GLINT_ERR_OUT_OF_MEMORY;
    }
    cudaMemcpy(g->d_params, params, sizeof(tg_params), cudaMemcpyHostToDevice);
    cudaMemcpy(g->d_objects, objects, sizeof(tg_object) * (size_t)num_objects, cudaMemcpyHostToDevice);
    *out = g;
    return cudaGetLastError() == cudaSuccess ? GLINT_OK : GLINT_ERR_CUDA;
}

glint_status glint_gen_step(glint_gen *g, double *d_out, void *stream) {
    if (!g || !d_out) return GLINT_ERR_INVALID_ARGUMENT;
    unsigned grid = glint::grid_for(g->n, 256, 152u * 16u);
    k_gen_step<<<grid, 256, 0, (cudaStream_t)stream>>>(g->d_params, g->d_objects, g->n, g->step, d_out);
    g->step++;
    return cudaGetLastError() == cudaSuccess ? GLINT_OK : GLINT_ERR_CUDA;
}

glint_status glint_gen_destroy(glint_gen *g) {
    if (!g) return GLINT_OK;
    cudaFree(g->d_params);
    cudaFree(g->d_objects);
    delete g;
    return GLINT_OK;
}

} /* extern "C" */
