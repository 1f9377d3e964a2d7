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
    const uint32_t nwork = a.cnt->n_leaf_work;
    const uint32_t tag = a.cnt->step_tag;
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(&a.cnt->work_next, 1u);
        li = __shfl_sync(0xffffffffu, li, 0);
        if (li >= nwork) break;
        const uint32_t g = a.work[li];
        const uint32_t s0 = a.grid_start[g];
        const uint32_t cnt_g = a.grid_count[g];
        const uint32_t k = cnt_g < cap ? cnt_g : cap;
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
        /* inside checks: p1 = member i, p2 = member j > i */
        for (uint32_t i = 0; i + 1 < k; ++i) {
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
        /* cross-leaf checks that target this leaf: p1 = the querier */
        const uint32_t tb = a.tstart[g], te = a.tstart[g + 1];
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

void refine_prec_set_attributes(uint32_t cap) {
    cudaFuncSetAttribute(k_refine_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)refine_prec_smem_bytes(cap));
}

} // namespace glint
