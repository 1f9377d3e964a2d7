/*
 * k_precision.cu -- the precision form of the refine stage: every candidate
 * pair is first screened in FP32 on exact fixed-point coordinate differences
 * (the Frame of glint_device.cuh), and only the pairs whose screened squared
 * distance lies inside the guard band around r^2 are re-tested with the
 * reference's FP64 arithmetic (point_le_exact), so the contact set - and every
 * meeting - stays identical to the reference's.
 *
 * The reference's test (tracing/refinement.cpp:19-31 with Point::distance,
 * geometry/geometry.h:40-48) divides the longitude difference by L(y1) of the
 * checking object; the screen multiplies the integer difference by that
 * object's cx = 1/(L(y1) S).  No FP64 instruction runs per pair outside the
 * band: on sm_103a FP64 issues at a small fraction of the FP32 rate.
 */
#include <cstring>

#include <atomic>

#include "refine_common.cuh"

namespace glint {

constexpr int kPrecWarps = 4;

/* one screened test; p1 scale cx, p2 scale c2 (a NaN in either forces the
 * exact path) */
__device__ inline int screen_pair(long long dx, long long dy, float cx, float c2, const Frame &f) {
    const Screen s = make_screen(__fmaf_rn(0.0f, c2, cx), f);
    return fx_screen(dx, dy, s, f.cy);
}

__global__ void __launch_bounds__(32 * kPrecWarps) k_refine_fp32(RefineArgs a) {
    extern __shared__ unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t cap = a.cap;
    /* per warp: X Y (i64), cx fx fy (f32), id (u32), queue */
    const size_t per_warp = (size_t)cap * 32 + sizeof(QEntry) * kQueue + 64;
    unsigned char *base = smem_raw + (size_t)w * ((per_warp + 63) & ~(size_t)63);
    long long *sX = reinterpret_cast<long long *>(base);
    long long *sY = sX + cap;
    float *sC = reinterpret_cast<float *>(sY + cap);
    float *sFx = sC + cap;
    float *sFy = sFx + cap;
    uint32_t *sid = reinterpret_cast<uint32_t *>(sFy + cap);
    QEntry *Q = reinterpret_cast<QEntry *>(((uintptr_t)(sid + cap) + 15) & ~(uintptr_t)15);
    const Frame f = a.f;

    unsigned long long cand = 0, hits = 0;
    uint32_t band = 0;
    uint32_t qn = 0;
    const uint32_t nwork = a.cnt->n_leaf_work, n_extra = a.cnt->n_extra;
    const uint32_t tag = a.cnt->step_tag;
    bool extra_done = n_extra == 0;
    uint32_t staged = ~0u;
    for (;;) {
        uint32_t g, chunk;
        if (!claim_item(a, nwork, n_extra, extra_done, g, chunk)) break;
        const uint32_t s0 = a.grid_start[g];
        const uint32_t cnt_g = a.grid_count[g];
        const uint32_t k = cnt_g < cap ? cnt_g : cap;
        if (g != staged) {
            for (uint32_t i = lane; i < k; i += 32) {
                const longlong2 ip = a.sipos[s0 + i];
                const float2 fp = a.sfpos[s0 + i];
                sX[i] = ip.x;
                sY[i] = ip.y;
                sC[i] = a.sc[s0 + i];
                sFx[i] = fp.x;
                sFy[i] = fp.y;
                sid[i] = a.sorted[s0 + i];
            }
            __syncwarp();
            staged = g;
        }
        /* inside checks: p1 = member i, p2 = member j > i */
        for (uint32_t i = 0; chunk == 0 && i + 1 < k; ++i) {
            const long long Xi = sX[i], Yi = sY[i];
            const float ci = sC[i];
            const uint32_t p1 = sid[i];
            for (uint32_t jb = i + 1; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long pw = 0;
                if (j < k) {
                    ++cand;
                    int r = screen_pair(Xi - sX[j], Yi - sY[j], ci, sC[j], f);
                    if (r < 0) {
                        ++band;
                        const double2 P = a.sxy[s0 + i], Q2 = a.sxy[s0 + j];
                        r = point_le_exact(P.x, P.y, Q2.x, Q2.y, dpm_lon_fast(P.y), a.ex) ? 1 : 0;
                    }
                    hit = r == 1;
                    if (hit) {
                        ++hits;
                        pw = pair_word(p1, sid[j]);
                    }
                }
                enqueue(a, Q, qn, hit, pw, prio_pack(0, p1, 0, j), sFx[i], sFy[i], hit ? sFx[j] : 0.f,
                        hit ? sFy[j] : 0.f, tag);
            }
        }
        /* cross-leaf checks that target this leaf, this item's chunk: p1 = the
         * querier */
        uint32_t tb, te;
        item_checks(a, g, chunk, tb, te);
        for (uint32_t t = tb; t < te; ++t) {
            const uint2 qe = a.tlist[t];
            const uint32_t q = qe.x;
            const uint32_t qr = a.rank_of[q];
            const longlong2 qi = a.sipos[qr];
            const float cq = a.sc[qr];
            const float2 qf = a.sfpos[qr];
            const uint32_t qgid = a.obj_gid[q];
            const bool qstored = (qr - a.grid_start[qgid]) < cap;
            for (uint32_t jb = 0; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long pw = 0;
                if (j < k) {
                    ++cand;
                    const long long dx = qi.x - sX[j], dy = qi.y - sY[j];
                    int r = screen_pair(dx, dy, cq, sC[j], f);
                    if (r < 0) {
                        ++band;
                        const double2 P = a.sxy[qr], M = a.sxy[s0 + j];
                        r = point_le_exact(P.x, P.y, M.x, M.y, dpm_lon_fast(P.y), a.ex) ? 1 : 0;
                    }
                    hit = r == 1;
                    if (hit) {
                        ++hits;
                        const uint32_t m = sid[j];
                        /* the same pair tested from m's side comes first in the
                         * reference's order when m < q; keep only one event */
                        if (q > m && qstored && has_check(a, m, qgid)) {
                            int r2 = screen_pair(dx, dy, sC[j], cq, f);
                            if (r2 < 0) {
                                ++band;
                                const double2 P = a.sxy[qr], M = a.sxy[s0 + j];
                                r2 = point_le_exact(M.x, M.y, P.x, P.y, dpm_lon_fast(M.y), a.ex) ? 1 : 0;
                            }
                            if (r2 == 1) hit = false;
                        }
                        if (hit) pw = pw_of(q, m);
                    }
                }
                enqueue(a, Q, qn, hit, pw, prio_pack(1, q, qe.y, j), qf.x, qf.y, hit ? sFx[j] : 0.f,
                        hit ? sFy[j] : 0.f, tag);
            }
        }
        __syncwarp();
    }
    drain_queue(a, Q, qn, tag);
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_down_sync(0xffffffffu, cand, o);
        hits += __shfl_down_sync(0xffffffffu, hits, o);
        band += __shfl_down_sync(0xffffffffu, band, o);
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->candidates, cand);
        atomicAdd(&a.cnt->contacts, hits);
        if (band) atomicAdd(&a.cnt->band_pairs, band);
    }
}

size_t refine_prec_smem_bytes(uint32_t cap) {
    const size_t per_warp = (size_t)cap * 32 + sizeof(QEntry) * kQueue + 64;
    return (size_t)kPrecWarps * ((per_warp + 63) & ~(size_t)63);
}

cudaError_t launch_refine_precision(glint_ctx *c, const RefineArgs &a) {
    k_refine_fp32<<<152 * 8, 32 * kPrecWarps, refine_prec_smem_bytes(c->cap), c->stream>>>(a);
    return cudaGetLastError();
}

/* as refine_set_attributes: the limit only grows (it is per kernel, not
 * per context) */
void refine_prec_set_attributes(uint32_t cap) {
    static std::atomic<uint32_t> largest{0};
    uint32_t m = largest.load();
    while (cap > m && !largest.compare_exchange_weak(m, cap)) {
    }
    const uint32_t use = cap > m ? cap : m;
    cudaFuncSetAttribute(k_refine_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)refine_prec_smem_bytes(use));
}

/* ---- probe: the screen against the FP64 test on sampled pairs --------------
 * Pairs (i, i + o), o = 1..32, for leaf-major ranks i = 0, stride, 2 stride,
 * ...: neighbours in that order share a leaf or sit in adjacent leaves, so the
 * sample is dominated by short distances, where the decision is made. */
struct ProbeAcc {
    unsigned long long pairs, in_band, mismatches, contacts;
    unsigned long long err_bits, err_near_bits, band_bits; /* non-negative doubles as bits */
};

__device__ inline unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ inline unsigned long long warp_max(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

__global__ void __launch_bounds__(256) k_precision_probe(const longlong2 *__restrict__ sipos,
                                                         const double2 *__restrict__ sxy,
                                                         const float *__restrict__ sc, uint32_t N, uint32_t stride,
                                                         Frame f, ExactCtx ex, ProbeAcc *acc) {
    const unsigned long long samples = ((unsigned long long)N + stride - 1) / stride;
    const unsigned long long total = samples * 32;
    unsigned long long pairs = 0, band = 0, mism = 0, hits = 0;
    double err = 0.0, err_near = 0.0, bandm = 0.0;
    const double r = ex.r;
    const unsigned long long step = (unsigned long long)gridDim.x * blockDim.x;
    /* every lane runs the same number of iterations (the warp reductions
     * below need all 32) */
    const unsigned long long start = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    for (unsigned long long it0 = start - (threadIdx.x & 31); it0 < total; it0 += step) {
        const unsigned long long it = it0 + (threadIdx.x & 31);
        const unsigned long long i = (it >> 5) * stride, j = i + (it & 31) + 1;
        if (it >= total || j >= N) continue;
        ++pairs;
        const longlong2 a = sipos[i], b = sipos[j];
        const float ci = sc[i], cj = sc[j];
        const long long dx = a.x - b.x, dy = a.y - b.y;
        const Screen s = make_screen(__fmaf_rn(0.0f, cj, ci), f);
        const int scr = fx_screen(dx, dy, s, f.cy);
        const double2 P = sxy[i], Q = sxy[j];
        const bool within = point_le_exact(P.x, P.y, Q.x, Q.y, dpm_lon_fast(P.y), ex);
        hits += within ? 1 : 0;
        if (scr < 0) ++band;
        else if ((scr == 1) != within) ++mism;
        const float mx = fx_to_f(dx) * s.cx, my = fx_to_f(dy) * f.cy;
        const float d32 = sqrtf(mx * mx + my * my);
        if (d32 == d32) {
            const double d64 = point_dist(P.x, P.y, Q.x, Q.y, dpm_lon_fast(P.y), ex.dpm_lat);
            const double e = fabs((double)d32 - d64);
            err = fmax(err, e);
            if (d64 <= 2.0 * r) err_near = fmax(err_near, e);
            const double bw = (double)(f.band0 + f.band1 * (s.cx + f.cy)) / (2.0 * r);
            if (bw == bw) bandm = fmax(bandm, bw);
        }
    }
    pairs = warp_sum(pairs);
    band = warp_sum(band);
    mism = warp_sum(mism);
    hits = warp_sum(hits);
    const unsigned long long eb = warp_max((unsigned long long)__double_as_longlong(err));
    const unsigned long long enb = warp_max((unsigned long long)__double_as_longlong(err_near));
    const unsigned long long bb = warp_max((unsigned long long)__double_as_longlong(bandm));
    if ((threadIdx.x & 31) == 0 && pairs) {
        atomicAdd(&acc->pairs, pairs);
        atomicAdd(&acc->in_band, band);
        atomicAdd(&acc->mismatches, mism);
        atomicAdd(&acc->contacts, hits);
        atomicMax(&acc->err_bits, eb);
        atomicMax(&acc->err_near_bits, enb);
        atomicMax(&acc->band_bits, bb);
    }
}

} // namespace glint

using namespace glint;

extern "C" glint_status glint_precision_probe(glint_ctx *c, uint32_t stride, glint_precision_report *out) {
    if (!c || !out || stride == 0) return GLINT_ERR_INVALID_ARGUMENT;
    if (c->step_index == 0) {
        c->last_error = "precision probe before the first step";
        return GLINT_ERR_STATE;
    }
    cudaSetDevice(c->device);
    ProbeAcc *d = nullptr;
    ProbeAcc h;
    std::memset(&h, 0, sizeof(h));
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d, sizeof(ProbeAcc));
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(ProbeAcc), c->stream);
    if (e == cudaSuccess) {
        ExactCtx ex = make_exact(c);
        ex.ambiguous = nullptr; /* the step's counters stay the step's */
        ex.rechecks = nullptr;
        const unsigned long long total = (((unsigned long long)c->N + stride - 1) / stride) * 32;
        k_precision_probe<<<grid_for(total, 256, 152u * 8u), 256, 0, c->stream>>>(c->d_sipos, c->d_sxy, c->d_sc,
                                                                                 c->N, stride, c->frame, ex, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (d) cudaFree(d);
    if (e != cudaSuccess) {
        c->last_error = std::string("precision probe: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    std::memset(out, 0, sizeof(*out));
    out->pairs = h.pairs;
    out->in_band = h.in_band;
    out->mismatches = h.mismatches;
    out->contacts = h.contacts;
    std::memcpy(&out->max_abs_err_m, &h.err_bits, sizeof(double));
    std::memcpy(&out->max_abs_err_near_m, &h.err_near_bits, sizeof(double));
    std::memcpy(&out->max_band_m, &h.band_bits, sizeof(double));
    out->stride = stride;
    return GLINT_OK;
}
