/*
 * k_precision.cu -- the precision form of the refine stage: candidate pairs
 * are first tested in FP32 on coordinates relative to the leaf, and only the
 * pairs whose FP32 distance lies inside a guard band around the reach are
 * re-tested with the reference's exact FP64 arithmetic (point_le_exact), so
 * the contact set - and every meeting - stays identical to the reference's.
 *
 * Guard band.  For a tile with origin o (its first member), each object keeps
 * u = fl32(x - o.x), v = fl32(y - o.y) (degrees; the FP64 subtraction is exact
 * for nearby longitudes) and iL = fl32(1/L(y)).  For a pair with p1 = i the
 * reference decides sqrt(X^2 + Y^2) <= r with X = (x_i - x_j)/L_i and
 * Y = (y_i - y_j)/dpm_lat (geometry/geometry.h:40-48).  With unit roundoff
 * u = 2^-24 the FP32 values fx = (u_i - u_j) iL_i, fy = (v_i - v_j) iM obey
 *   |fx - X| <= u (3|X| + 2 (|u_i| + |u_j|) iL_i),   likewise for fy,
 * and near the threshold (|X|, |Y| <= r) the FP32 square q = fx^2 + fy^2 obeys
 *   |q - (X^2 + Y^2)| <= u (16 r^2 + 4 r W)
 * where W = (|u_i| + |u_j|) iL_i + (|v_i| + |v_j|) iM is the pair's offset
 * size in metres.  The band is twice that; outside it the FP32 decision equals
 * the reference's (the FP64 rounding of the reference is ~2^-50 relative).
 */
#include "refine_common.cuh"

namespace glint {

constexpr int kPrecWarps = 4;

struct PrecParams {
    float r2;        /* r^2 */
    float iMf;       /* 1 / dpm_lat */
    float band_k0;   /* 2 * 2^-24 * 16 r^2 */
    float band_k1;   /* 2 * 2^-24 * 4 r */
};

__device__ inline int prec_test(float du, float dv, float iL, float w_m, const PrecParams &pp) {
    const float fx = du * iL, fy = dv * pp.iMf;
    const float q = fx * fx + fy * fy;
    const float band = pp.band_k0 + pp.band_k1 * w_m;
    if (q < pp.r2 - band) return 1;
    if (q > pp.r2 + band) return 0;
    return -1; /* inside the guard band: decide exactly */
}

__global__ void __launch_bounds__(32 * kPrecWarps) k_refine_fp32(RefineArgs a, PrecParams pp) {
    extern __shared__ unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t cap = a.cap;
    /* per warp: x y L (double), u v iL (float), id (u32), queue */
    const size_t per_warp = (size_t)cap * 40 + sizeof(QEntry) * kQueue + 64;
    unsigned char *base = smem_raw + (size_t)w * ((per_warp + 63) & ~(size_t)63);
    double *sx = reinterpret_cast<double *>(base);
    double *sy = sx + cap;
    double *sLm = sy + cap;
    float *su = reinterpret_cast<float *>(sLm + cap);
    float *sv = su + cap;
    float *siL = sv + cap;
    uint32_t *sid = reinterpret_cast<uint32_t *>(siL + cap);
    QEntry *Q = reinterpret_cast<QEntry *>(((uintptr_t)(sid + cap) + 15) & ~(uintptr_t)15);

    unsigned long long cand = 0, hits = 0;
    uint32_t band = 0;
    uint32_t qn = 0;
    const uint32_t nwork = a.cnt->n_leaf_work;
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(&a.cnt->work_next, 1u);
        li = __shfl_sync(0xffffffffu, li, 0);
        if (li >= nwork) break;
        const uint32_t g = a.work[li];
        const uint32_t s0 = a.grid_start[g];
        const uint32_t cnt_g = a.grid_count[g];
        const uint32_t k = cnt_g < cap ? cnt_g : cap;
        const double2 org = a.sxy[s0];
        for (uint32_t i = lane; i < k; i += 32) {
            const double2 p = a.sxy[s0 + i];
            const double L = a.sL[s0 + i];
            sx[i] = p.x;
            sy[i] = p.y;
            sLm[i] = L;
            su[i] = (float)(p.x - org.x);
            sv[i] = (float)(p.y - org.y);
            siL[i] = (float)(1.0 / L);
            sid[i] = a.sorted[s0 + i];
        }
        __syncwarp();
        for (uint32_t i = 0; i + 1 < k; ++i) {
            const float ui = su[i], vi = sv[i], iLi = siL[i];
            const float aui = fabsf(ui), avi = fabsf(vi);
            const uint32_t p1 = sid[i];
            for (uint32_t jb = i + 1; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long pw = 0;
                float fx1 = 0.f, fy1 = 0.f, fx2 = 0.f, fy2 = 0.f;
                if (j < k) {
                    ++cand;
                    const float uj = su[j], vj = sv[j];
                    const float wm = (aui + fabsf(uj)) * iLi + (avi + fabsf(vj)) * pp.iMf;
                    int r = prec_test(ui - uj, vi - vj, iLi, wm, pp);
                    if (r < 0) {
                        ++band;
                        r = point_le_exact(sx[i], sy[i], sx[j], sy[j], sLm[i], a.ex) ? 1 : 0;
                    }
                    hit = r == 1;
                    if (hit) {
                        ++hits;
                        pw = pair_word(p1, sid[j]);
                        fx1 = (float)sx[i];
                        fy1 = (float)sy[i];
                        fx2 = (float)sx[j];
                        fy2 = (float)sy[j];
                    }
                }
                enqueue(a, Q, qn, hit, pw, prio_pack(0, p1, 0, j), fx1, fy1, fx2, fy2);
            }
        }
        const uint32_t tb = a.tstart[g], te = a.tstart[g + 1];
        for (uint32_t t = tb; t < te; ++t) {
            const uint2 qe = a.tlist[t];
            const uint32_t q = qe.x;
            const double2 qp = a.pts[q];
            const double Lq = a.L[q];
            const uint32_t qgid = a.obj_gid[q];
            const bool qstored = (a.rank_of[q] - a.grid_start[qgid]) < cap;
            const float uq = (float)(qp.x - org.x), vq = (float)(qp.y - org.y), iLq = (float)(1.0 / Lq);
            const float auq = fabsf(uq), avq = fabsf(vq);
            for (uint32_t jb = 0; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long pw = 0;
                float fx2 = 0.f, fy2 = 0.f;
                if (j < k) {
                    ++cand;
                    const float uj = su[j], vj = sv[j];
                    const float auj = fabsf(uj), avj = fabsf(vj);
                    int r = prec_test(uq - uj, vq - vj, iLq, (auq + auj) * iLq + (avq + avj) * pp.iMf, pp);
                    if (r < 0) {
                        ++band;
                        r = point_le_exact(qp.x, qp.y, sx[j], sy[j], Lq, a.ex) ? 1 : 0;
                    }
                    hit = r == 1;
                    if (hit) {
                        ++hits;
                        const uint32_t m = sid[j];
                        if (q > m && qstored && has_check(a, m, qgid)) {
                            /* the mirrored test, p1 = m */
                            int r2 = prec_test(uj - uq, vj - vq, siL[j], (auq + auj) * siL[j] + (avq + avj) * pp.iMf, pp);
                            if (r2 < 0) {
                                ++band;
                                r2 = point_le_exact(sx[j], sy[j], qp.x, qp.y, sLm[j], a.ex) ? 1 : 0;
                            }
                            if (r2 == 1) hit = false;
                        }
                        if (hit) {
                            pw = pw_of(q, m);
                            fx2 = (float)sx[j];
                            fy2 = (float)sy[j];
                        }
                    }
                }
                enqueue(a, Q, qn, hit, pw, prio_pack(1, q, qe.y, j), (float)qp.x, (float)qp.y, fx2, fy2);
            }
        }
        __syncwarp();
    }
    drain_queue(a, Q, qn);
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
    const size_t per_warp = (size_t)cap * 40 + sizeof(QEntry) * kQueue + 64;
    return (size_t)kPrecWarps * ((per_warp + 63) & ~(size_t)63);
}

cudaError_t launch_refine_precision(glint_ctx *c, const RefineArgs &a) {
    PrecParams pp;
    const double r = c->cfg.reach_distance;
    pp.r2 = (float)(r * r);
    pp.iMf = (float)(1.0 / c->dpm_lat);
    const double u = std::ldexp(1.0, -24);
    pp.band_k0 = (float)(2.0 * u * 16.0 * r * r);
    pp.band_k1 = (float)(2.0 * u * 4.0 * r);
    k_refine_fp32<<<152 * 8, 32 * kPrecWarps, refine_prec_smem_bytes(c->cap), c->stream>>>(a, pp);
    return cudaGetLastError();
}

void refine_prec_set_attributes(uint32_t cap) {
    cudaFuncSetAttribute(k_refine_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)refine_prec_smem_bytes(cap));
}

} // namespace glint
