/*
 * k_refine.cu -- stages (b) part 2, (c) and (d) part 1 in the plain form:
 * per-leaf candidate enumeration, the reference's FP64 distance test on every
 * candidate, and the meeting-table update.
 *
 * Candidates (tracing/refinement.cpp:19-31): for every check and every stored
 * member of its leaf with pid < member (inside checks) or any member
 * (cross-leaf checks).  p1 is the checking object, whose latitude sets
 * degree_per_meter_longitude in Point::distance (geometry/geometry.h:40-48).
 *
 * Device form: one warp per leaf.  The leaf's stored members (its first
 * min(count, capacity) objects in id order) are staged in shared memory as
 * SoA x / y / L / id; the warp runs the inside pairs i < j and then every
 * cross-leaf check that targets the leaf against the staged members.  Pairs
 * within reach go through the contact queue (refine_common.cuh): a pair found
 * in the table as it stood at the start of the step is touched there, which is
 * what the reference does for it; a pair not found goes to the new list with
 * its position in the reference's sequential check order as priority.
 *
 * Duplicate pairs: a cross-leaf pair (a, b) is tested from both sides when a
 * has a check on b's leaf and b one on a's leaf.  The reference's second test
 * only re-touches the entry the first one made; here the test from the larger
 * id is dropped when the other test also passes, so every pair has at most
 * one event per step.
 */
#include <algorithm>
#include <atomic>

#include "refine_common.cuh"

namespace glint {

constexpr int kRefineWarps = 4;

__global__ void __launch_bounds__(32 * kRefineWarps) k_refine_fp64(RefineArgs a) {
    extern __shared__ unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t cap = a.cap;
    /* per-warp layout: x[cap] y[cap] L[cap] (double), id[cap] (u32), queue */
    const size_t per_warp = (size_t)cap * 28 + sizeof(QEntry) * kQueue + 64;
    unsigned char *base = smem_raw + (size_t)w * ((per_warp + 63) & ~(size_t)63);
    double *sx = reinterpret_cast<double *>(base);
    double *sy = sx + cap;
    double *sLm = sy + cap;
    uint32_t *sid = reinterpret_cast<uint32_t *>(sLm + cap);
    QEntry *Q = reinterpret_cast<QEntry *>(((uintptr_t)(sid + cap) + 15) & ~(uintptr_t)15);

    unsigned long long cand = 0, hits = 0;
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
                const double2 p = a.sxy[s0 + i];
                sx[i] = p.x;
                sy[i] = p.y;
                sLm[i] = a.sL[s0 + i];
                sid[i] = a.sorted[s0 + i];
            }
            __syncwarp();
            staged = g;
        }
        /* inside checks: p1 = member i, p2 = member j > i (ids ascend with rank) */
        for (uint32_t i = 0; chunk == 0 && i + 1 < k; ++i) {
            const double x1 = sx[i], y1 = sy[i], L1 = sLm[i];
            const uint32_t p1 = sid[i];
            const float fx1 = (float)x1, fy1 = (float)y1;
            for (uint32_t jb = i + 1; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long pw = 0;
                float fx2 = 0.f, fy2 = 0.f;
                if (j < k) {
                    ++cand;
                    const double x2 = sx[j], y2 = sy[j];
                    hit = point_le_exact(x1, y1, x2, y2, L1, a.ex);
                    if (hit) {
                        ++hits;
                        pw = pair_word(p1, sid[j]);
                        fx2 = (float)x2;
                        fy2 = (float)y2;
                    }
                }
                enqueue(a, Q, qn, hit, pw, prio_pack(0, p1, 0, j), fx1, fy1, fx2, fy2, tag);
            }
        }
        /* cross-leaf checks that target this leaf: this item's chunk */
        uint32_t tb, te;
        item_checks(a, g, chunk, tb, te);
        for (uint32_t t = tb; t < te; ++t) {
            const uint2 qe = a.tlist[t];
            const uint32_t q = qe.x;
            const uint32_t qr = a.rank_of[q];
            const double2 qp = a.sxy[qr];
            const double Lq = a.sL[qr];
            const uint32_t qgid = a.obj_gid[q];
            const bool qstored = (qr - a.grid_start[qgid]) < cap;
            const float fqx = (float)qp.x, fqy = (float)qp.y;
            for (uint32_t jb = 0; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long pw = 0;
                float fx2 = 0.f, fy2 = 0.f;
                if (j < k) {
                    ++cand;
                    const double x2 = sx[j], y2 = sy[j];
                    hit = point_le_exact(qp.x, qp.y, x2, y2, Lq, a.ex);
                    if (hit) {
                        ++hits;
                        const uint32_t m = sid[j];
                        /* the same pair tested from m's side comes first in the
                         * reference's order when m < q; keep only one event */
                        if (q > m && qstored && has_check(a, m, qgid) && point_le_exact(x2, y2, qp.x, qp.y, sLm[j], a.ex))
                            hit = false;
                        if (hit) {
                            pw = pw_of(q, m);
                            fx2 = (float)x2;
                            fy2 = (float)y2;
                        }
                    }
                }
                enqueue(a, Q, qn, hit, pw, prio_pack(1, q, qe.y, j), fqx, fqy, fx2, fy2, tag);
            }
        }
        __syncwarp();
    }
    drain_queue(a, Q, qn, tag);
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_down_sync(0xffffffffu, cand, o);
        hits += __shfl_down_sync(0xffffffffu, hits, o);
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->candidates, cand);
        atomicAdd(&a.cnt->contacts, hits);
    }
}

/* shared memory per warp (its leaf's members and its contact queue), and the
 * warps per block that fit the per-block limit (large leaf buffers run with
 * fewer warps per block) */
static size_t refine_warp_bytes(uint32_t cap) {
    const size_t per_warp = (size_t)cap * 28 + sizeof(QEntry) * kQueue + 64;
    return (per_warp + 63) & ~(size_t)63;
}
int refine_warps(uint32_t cap) {
    return (int)std::max<size_t>(1, std::min<size_t>(kRefineWarps, kMaxBlockSmem / refine_warp_bytes(cap)));
}
size_t refine_smem_bytes(uint32_t cap) { return (size_t)refine_warps(cap) * refine_warp_bytes(cap); }

/* the chunks beyond the first of every leaf's cross-leaf checks */
__global__ void __launch_bounds__(256) k_refine_extra(const uint32_t *__restrict__ work,
                                                      const uint32_t *__restrict__ tstart, uint2 *__restrict__ extra,
                                                      uint64_t cap, uint32_t per_item, DevCounters *cnt) {
    const uint32_t nwork = cnt->n_leaf_work;
    for (uint32_t li = blockIdx.x * blockDim.x + threadIdx.x; li < nwork; li += gridDim.x * blockDim.x) {
        const uint32_t g = work[li];
        const uint32_t cross = tstart[g + 1] - tstart[g];
        const uint32_t chunks = (cross + per_item - 1) / per_item;
        for (uint32_t ch = 1; ch < chunks; ++ch) {
            const uint32_t idx = atomicAdd(&cnt->n_extra, 1u);
            if (idx < cap) extra[idx] = make_uint2(g, ch);
            else atomicOr(&cnt->error_flags, GLINT_EF_CHECKS_OVERFLOW);
        }
    }
}

RefineArgs refine_args(glint_ctx *c) {
    RefineArgs a;
    a.work = c->d_leaf_work;
    a.grid_start = c->d_grid_start;
    a.grid_count = c->d_grid_count;
    a.sorted = c->d_sorted;
    a.sxy = c->d_sxy;
    a.sL = c->d_sL;
    a.tstart = c->d_tstart;
    a.tlist = c->d_tlist;
    a.sipos = c->d_sipos;
    a.sfpos = c->d_sfpos;
    a.sc = c->d_sc;
    a.f = c->frame;
    a.obj_gid = c->d_obj_gid;
    a.rank_of = c->d_rank_of;
    a.qstart = c->d_qstart;
    a.qlist = c->d_qlist;
    a.extra = c->d_rextra;
    a.tab = c->d_tab;
    a.stamp = c->d_stamp;
    a.newlist = c->d_new;
    a.B = c->B;
    a.Bm = c->Bm;
    a.new_cap = c->new_cap;
    a.cap = c->cap;
    a.chunk = c->chunk;
    a.extra_cap = (uint32_t)std::min<uint64_t>(c->rextra_cap, 0xffffffffu);
    a.ex = make_exact(c);
    a.cnt = c->d_cnt;
    return a;
}

cudaError_t launch_refine_precision(glint_ctx *c, const RefineArgs &a);

/* the refine stage's work items: each leaf's chunks beyond its first */
cudaError_t launch_refine_items(glint_ctx *c) {
    k_refine_extra<<<grid_for(c->G, 256), 256, 0, c->stream>>>(c->d_leaf_work, c->d_tstart, c->d_rextra,
                                                               c->rextra_cap, c->chunk, c->d_cnt);
    return cudaGetLastError();
}

/* the refine stage's pair tests over its work items */
cudaError_t launch_refine_pairs(glint_ctx *c) {
    RefineArgs a = refine_args(c);
    if (c->cfg.precision_mode == 1) return launch_refine_precision(c, a);
    k_refine_fp64<<<152 * 8, 32 * refine_warps(c->cap), refine_smem_bytes(c->cap), c->stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_refine(glint_ctx *c, uint32_t /*cur_time*/) {
    cudaError_t e = launch_refine_items(c);
    return e != cudaSuccess ? e : launch_refine_pairs(c);
}

/* The limit is a property of the kernel, shared by every context of the
 * process: it is set to the per-block maximum, and every launch asks for the
 * shared memory its leaf buffer needs. */
void refine_set_attributes(uint32_t cap) {
    (void)cap;
    cudaFuncSetAttribute(k_refine_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxBlockSmem);
}

/* ---- insertion of the step's new pairs -------------------------------------
 * Deterministic linear probing with priority displacement: a pair walking from
 * its home bucket takes an empty bucket, or swaps itself into a bucket held by
 * a pair inserted this step with a larger priority (which then walks on from
 * the next bucket).  Committed pairs are never moved.  The final layout is
 * the one a single thread produces by inserting the pairs one by one in
 * priority order, which is the reference's order (tracing/refinement.cpp:
 * 34-55).  A pair that meets its own committed entry further along (left there
 * when an earlier bucket of its probe run emptied) touches that entry instead,
 * as the reference does when its probe reaches it. */
__device__ inline bool u128_eq(const ulonglong2 &a, const ulonglong2 &b) { return a.x == b.x && a.y == b.y; }

__device__ inline ulonglong2 cas128(TRec *r, ulonglong2 expect, ulonglong2 desired) {
    unsigned __int128 e = ((unsigned __int128)expect.y << 64) | expect.x;
    unsigned __int128 d = ((unsigned __int128)desired.y << 64) | desired.x;
    unsigned __int128 o = atomicCAS(reinterpret_cast<unsigned __int128 *>(r), e, d);
    return make_ulonglong2((unsigned long long)o, (unsigned long long)(o >> 64));
}

__device__ inline void touch_box(TRec &r, const float2 &A, const float2 &Bp) {
    const float ax = A.x, ay = A.y, bx = Bp.x, by = Bp.y;
    uint4 m = *reinterpret_cast<const uint4 *>(r.mbr);
    m.x = min(m.x, min(fenc(ax), fenc(bx)));
    m.y = min(m.y, min(fenc(ay), fenc(by)));
    m.z = max(m.z, max(fenc(ax), fenc(bx)));
    m.w = max(m.w, max(fenc(ay), fenc(by)));
    *reinterpret_cast<uint4 *>(r.mbr) = m;
}

__global__ void __launch_bounds__(256) k_insert(const NewEntry *__restrict__ list, TRec *tab, uint32_t *newline,
                                                uint64_t B, uint64_t Bm, uint64_t new_cap,
                                                const float2 *__restrict__ fpos, uint32_t N,
                                                DevCounters *cnt) {
    const unsigned long long n0 = cnt->new_keys;
    const unsigned long long n = n0 < new_cap ? n0 : new_cap;
    const uint8_t st = (uint8_t)cnt->step_tag;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        ulonglong2 cur = make_ulonglong2(list[i].key | kNewFlag, list[i].prio);
        uint64_t slot = fastmod(cantor(pair_a(cur.x), pair_b(cur.x)), B, Bm);
        bool done = false;
        /* empty records hold (kEmptyW0, 0), so the first compare-and-swap at a
         * bucket doubles as its read */
        const ulonglong2 empty = make_ulonglong2(kEmptyW0, 0ull);
        for (uint32_t iter = 0; iter < kProbeLimit && !done; ++iter) {
            ulonglong2 seen = empty;
            for (uint32_t retry = 0;; ++retry) {
                if (retry >= kProbeLimit) {
                    atomicOr(&cnt->error_flags, GLINT_EF_TABLE_FULL);
                    done = true;
                    break;
                }
                const unsigned long long plain = cur.x & kPairMask;
                if (seen.x == kEmptyW0) {
                    ulonglong2 prev = cas128(&tab[slot], seen, cur);
                    if (u128_eq(prev, seen)) {
                        atomicOr(&newline[slot >> 7], 1u << ((slot >> 2) & 31));
                        done = true;
                        break;
                    }
                    seen = prev;
                    continue;
                }
                if (seen.x == plain) {
                    /* the carried pair's own committed entry */
                    const uint32_t pa = pair_a(plain), pb = pair_b(plain);
                    if (pa < N && pb < N) touch_box(tab[slot], fpos[pa], fpos[pb]);
                    rec_set_tag(tab[slot], st);
                    done = true;
                    break;
                }
                if (seen.x == cur.x) {
                    atomicOr(&cnt->error_flags, GLINT_EF_DUPLICATE_NEW);
                    done = true;
                    break;
                }
                if ((seen.x & kNewFlag) && seen.y > cur.y) {
                    ulonglong2 prev = cas128(&tab[slot], seen, cur);
                    if (u128_eq(prev, seen)) {
                        cur = seen; /* the displaced pair walks on */
                        break;
                    }
                    seen = prev;
                    continue;
                }
                break; /* a committed pair or an earlier new pair */
            }
            if (!done) slot = (slot + 1 == B) ? 0 : slot + 1;
        }
        if (!done) atomicOr(&cnt->error_flags, GLINT_EF_TABLE_FULL);
    }
}

cudaError_t launch_insert(glint_ctx *c, uint32_t cur_time) {
    (void)cur_time;
    /* many short blocks: a thread's walk can be long (probe runs,
     * displacements), and with one resident wave of long grid-stride loops
     * the slowest threads set the kernel's end; up to 152 x 128 blocks
     * balance it (5.4 against 7.7 ms at 10M objects), fewer for a small
     * context's new-pair capacity */
    const unsigned blocks = (unsigned)std::min<uint64_t>(152u * 128u, std::max<uint64_t>(152u, c->new_cap / 2048));
    k_insert<<<blocks, 256, 0, c->stream>>>(c->d_new, c->d_tab, c->d_newline, c->B, c->Bm, c->new_cap, c->d_fpos, c->N,
                                             c->d_cnt);
    return cudaGetLastError();
}

} // namespace glint
