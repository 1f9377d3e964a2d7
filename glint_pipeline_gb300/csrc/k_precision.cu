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
#include <algorithm>
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

/* one warp's shared memory: its leaf's members (X Y as i64; cx fx fy as f32;
 * id) and its contact queue */
struct PrecSmem {
    long long *sX, *sY;
    float *sC, *sFx, *sFy;
    uint32_t *sid;
    QEntry *Q;
};

__host__ __device__ inline size_t prec_warp_bytes(uint32_t cap) {
    const size_t per_warp = (size_t)cap * 32 + sizeof(QEntry) * kQueue + 64;
    return (per_warp + 63) & ~(size_t)63;
}

__device__ inline PrecSmem prec_smem(unsigned char *base, uint32_t cap) {
    PrecSmem m;
    m.sX = reinterpret_cast<long long *>(base);
    m.sY = m.sX + cap;
    m.sC = reinterpret_cast<float *>(m.sY + cap);
    m.sFx = m.sC + cap;
    m.sFy = m.sFx + cap;
    m.sid = reinterpret_cast<uint32_t *>(m.sFy + cap);
    m.Q = reinterpret_cast<QEntry *>(((uintptr_t)(m.sid + cap) + 15) & ~(uintptr_t)15);
    return m;
}

/* a warp's tests and contacts of one context, added to its totals on flush */
struct PrecTally {
    unsigned long long cand = 0, hits = 0;
    uint32_t band = 0;
};

/* warp-collective: the queued contacts into context a's table, and the
 * warp's counts into its totals */
__device__ inline void prec_flush(const RefineArgs &a, QEntry *Q, uint32_t &qn, uint32_t tag, PrecTally &t) {
    drain_queue(a, Q, qn, tag);
    qn = 0;
    for (int o = 16; o > 0; o >>= 1) {
        t.cand += __shfl_down_sync(0xffffffffu, t.cand, o);
        t.hits += __shfl_down_sync(0xffffffffu, t.hits, o);
        t.band += __shfl_down_sync(0xffffffffu, t.band, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&a.cnt->candidates, t.cand);
        atomicAdd(&a.cnt->contacts, t.hits);
        if (t.band) atomicAdd(&a.cnt->band_pairs, t.band);
    }
    t = PrecTally();
}

/* warp-collective: one work item (leaf g, chunk) of context a */
__device__ inline void prec_item(const RefineArgs &a, uint32_t g, uint32_t chunk, const PrecSmem &m,
                                 uint32_t &staged, PrecTally &t, uint32_t &qn, uint32_t tag) {
    const int lane = threadIdx.x & 31;
    const uint32_t cap = a.cap;
    const Frame &f = a.f;
    long long *sX = m.sX, *sY = m.sY;
    float *sC = m.sC, *sFx = m.sFx, *sFy = m.sFy;
    uint32_t *sid = m.sid;
    QEntry *Q = m.Q;
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
                ++t.cand;
                int r = screen_pair(Xi - sX[j], Yi - sY[j], ci, sC[j], f);
                if (r < 0) {
                    ++t.band;
                    const double2 P = a.sxy[s0 + i], Q2 = a.sxy[s0 + j];
                    r = point_le_exact(P.x, P.y, Q2.x, Q2.y, dpm_lon_fast(P.y), a.ex) ? 1 : 0;
                }
                hit = r == 1;
                if (hit) {
                    ++t.hits;
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
    for (uint32_t tt = tb; tt < te; ++tt) {
        const uint2 qe = a.tlist[tt];
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
                ++t.cand;
                const long long dx = qi.x - sX[j], dy = qi.y - sY[j];
                int r = screen_pair(dx, dy, cq, sC[j], f);
                if (r < 0) {
                    ++t.band;
                    const double2 P = a.sxy[qr], M = a.sxy[s0 + j];
                    r = point_le_exact(P.x, P.y, M.x, M.y, dpm_lon_fast(P.y), a.ex) ? 1 : 0;
                }
                hit = r == 1;
                if (hit) {
                    ++t.hits;
                    const uint32_t mm = sid[j];
                    /* the same pair tested from mm's side comes first in the
                     * reference's order when mm < q; keep only one event */
                    if (q > mm && qstored && has_check(a, mm, qgid)) {
                        int r2 = screen_pair(dx, dy, sC[j], cq, f);
                        if (r2 < 0) {
                            ++t.band;
                            const double2 P = a.sxy[qr], M = a.sxy[s0 + j];
                            r2 = point_le_exact(M.x, M.y, P.x, P.y, dpm_lon_fast(M.y), a.ex) ? 1 : 0;
                        }
                        if (r2 == 1) hit = false;
                    }
                    if (hit) pw = pw_of(q, mm);
                }
            }
            enqueue(a, Q, qn, hit, pw, prio_pack(1, q, qe.y, j), qf.x, qf.y, hit ? sFx[j] : 0.f,
                    hit ? sFy[j] : 0.f, tag);
        }
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32 * kPrecWarps) k_refine_fp32(RefineArgs a) {
    extern __shared__ unsigned char smem_raw[];
    const int w = threadIdx.x >> 5;
    const PrecSmem m = prec_smem(smem_raw + (size_t)w * prec_warp_bytes(a.cap), a.cap);
    PrecTally t;
    uint32_t qn = 0;
    const uint32_t nwork = a.cnt->n_leaf_work, n_extra = a.cnt->n_extra;
    const uint32_t tag = a.cnt->step_tag;
    bool extra_done = n_extra == 0;
    uint32_t staged = ~0u;
    for (;;) {
        uint32_t g, chunk;
        if (!claim_item(a, nwork, n_extra, extra_done, g, chunk)) break;
        prec_item(a, g, chunk, m, staged, t, qn, tag);
    }
    prec_flush(a, m.Q, qn, tag, t);
}

/* ---- the refine stage of many contexts in one launch ---------------------
 * The items of all regions form one list: every region's extra chunks (the
 * long work) first, then every region's leaves.  A warp takes the next item,
 * finds its region, and works on it with that region's arguments, which it
 * keeps in its shared memory; before it moves to another region it drains
 * its queued contacts into the region it leaves.  Every contact carries its
 * place in the reference's order, so results do not depend on who tests it. */
__global__ void k_refine_batch_prep(const RefineArgs *__restrict__ args, uint32_t R, uint32_t *ex_off,
                                    uint32_t *wk_off, unsigned int *next) {
    uint32_t e = 0, w = 0;
    for (uint32_t r = 0; r < R; ++r) {
        ex_off[r] = e;
        wk_off[r] = w;
        const uint32_t ne = args[r].cnt->n_extra;
        e += ne < args[r].extra_cap ? ne : args[r].extra_cap;
        w += args[r].cnt->n_leaf_work;
    }
    ex_off[R] = e;
    wk_off[R] = w;
    *next = 0;
}

__device__ inline uint32_t region_of(const uint32_t *off, uint32_t R, uint32_t v) {
    uint32_t lo = 0, hi = R; /* off[lo] <= v < off[lo + 1] */
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (off[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(32 * kPrecWarps) k_refine_fp32_batch(const RefineArgs *__restrict__ args, uint32_t R,
                                                                       const uint32_t *__restrict__ ex_off,
                                                                       const uint32_t *__restrict__ wk_off,
                                                                       unsigned int *next, uint32_t cap_max) {
    extern __shared__ unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t kArgBytes = (sizeof(RefineArgs) + 63) & ~(size_t)63;
    unsigned char *base = smem_raw + (size_t)w * (kArgBytes + prec_warp_bytes(cap_max));
    RefineArgs *sa = reinterpret_cast<RefineArgs *>(base);
    const PrecSmem m = prec_smem(base + kArgBytes, cap_max);
    const uint32_t E = ex_off[R], W = wk_off[R];
    PrecTally t;
    uint32_t qn = 0, tag = 0, staged = ~0u, cur = ~0u;
    for (;;) {
        uint32_t v = 0;
        if (lane == 0) v = atomicAdd(next, 1u);
        v = __shfl_sync(0xffffffffu, v, 0);
        if (v >= E + W) break;
        uint32_t r, g, chunk;
        if (v < E) {
            r = region_of(ex_off, R, v);
            const uint2 e = args[r].extra[v - ex_off[r]];
            g = e.x;
            chunk = e.y;
        } else {
            r = region_of(wk_off, R, v - E);
            g = args[r].work[v - E - wk_off[r]];
            chunk = 0;
        }
        if (r != cur) {
            if (cur != ~0u) prec_flush(*sa, m.Q, qn, tag, t);
            __syncwarp();
            static_assert(sizeof(RefineArgs) % 4 == 0, "RefineArgs words");
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&args[r]);
            uint32_t *dst = reinterpret_cast<uint32_t *>(sa);
            for (uint32_t i = lane; i < sizeof(RefineArgs) / 4; i += 32) dst[i] = src[i];
            __syncwarp();
            cur = r;
            staged = ~0u;
            tag = sa->cnt->step_tag;
        }
        prec_item(*sa, g, chunk, m, staged, t, qn, tag);
    }
    if (cur != ~0u) prec_flush(*sa, m.Q, qn, tag, t);
}

int refine_prec_warps(uint32_t cap) {
    return (int)std::max<size_t>(1, std::min<size_t>(kPrecWarps, kMaxBlockSmem / prec_warp_bytes(cap)));
}

size_t refine_prec_smem_bytes(uint32_t cap) { return (size_t)refine_prec_warps(cap) * prec_warp_bytes(cap); }

cudaError_t launch_refine_precision(glint_ctx *c, const RefineArgs &a) {
    k_refine_fp32<<<152 * 8, 32 * refine_prec_warps(c->cap), refine_prec_smem_bytes(c->cap), c->stream>>>(a);
    return cudaGetLastError();
}

/* the refine pairs of R contexts in one launch on stream s; args, ex_off,
 * wk_off (R + 1 each) and next are device buffers of the caller */
cudaError_t launch_refine_precision_batch(const RefineArgs *d_args, uint32_t R, uint32_t cap_max, uint32_t *ex_off,
                                          uint32_t *wk_off, unsigned int *next, cudaStream_t s) {
    k_refine_batch_prep<<<1, 1, 0, s>>>(d_args, R, ex_off, wk_off, next);
    constexpr size_t kArgBytes = (sizeof(RefineArgs) + 63) & ~(size_t)63;
    const size_t per_warp = kArgBytes + prec_warp_bytes(cap_max);
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(kPrecWarps, kMaxBlockSmem / per_warp));
    k_refine_fp32_batch<<<152 * 8, 32 * warps, warps * per_warp, s>>>(d_args, R, ex_off, wk_off, next, cap_max);
    return cudaGetLastError();
}

/* the per-kernel limit, set to the per-block maximum: every launch asks for
 * the shared memory its leaf buffer needs */
void refine_prec_set_attributes(uint32_t cap) {
    (void)cap;
    cudaFuncSetAttribute(k_refine_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxBlockSmem);
    cudaFuncSetAttribute(k_refine_fp32_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxBlockSmem);
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
