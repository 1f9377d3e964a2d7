/*
 * k_refine.cu -- stages (b) part 2, (c) and (d) part 1: per-leaf candidate
 * enumeration, the exact distance test, and the meeting-table update.
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
 * within reach are compacted with a warp ballot into a shared queue and
 * processed 32 at a time:
 *   - the pair's key is looked up from its home slot in the table as it was
 *     at the start of the step (no keys change during this kernel); if found
 *     before an empty slot the entry is touched (stamp, f32 box), which is
 *     exactly what the reference does for it;
 *   - otherwise (key, priority) goes to the new list, inserted by k_insert.
 * The priority is the event's position in the reference's sequential check
 * order, so the insertion can reproduce the reference's slot placement.
 *
 * Duplicate pairs: a cross-leaf pair (a, b) is tested from both sides when a
 * has a check on b's leaf and b one on a's leaf.  The reference handles the
 * second test as a hit on the first one's entry; here the event with the
 * larger priority is dropped when the other test also passes, so every new
 * key enters the new list once.
 */
#include "glint_internal.cuh"

namespace glint {

constexpr int kRefineWarps = 4;
constexpr int kQueue = 64;
constexpr uint32_t kProbeLimit = 1u << 22;

struct QEntry {
    unsigned long long key;
    unsigned long long prio;
    float x1, y1, x2, y2;
};

struct RefineArgs {
    const uint32_t *work;
    const uint32_t *grid_start;
    const uint32_t *grid_count;
    const uint32_t *sorted;
    const double2 *sxy;
    const double *sL;
    const uint32_t *tstart;
    const uint2 *tlist;
    const double2 *pts;
    const double *L;
    const uint32_t *obj_gid;
    const uint32_t *rank_of;
    const uint32_t *qstart;
    const uint32_t *qlist;
    TRec *tab;
    uint8_t *stamp;
    NewEntry *newlist;
    uint64_t B, Bm, new_cap;
    uint32_t cap;
    uint8_t st;
    ExactCtx ex;
    DevCounters *cnt;
};

/* look the key up in the table as it stood at the start of the step */
__device__ inline bool table_touch(const RefineArgs &a, const QEntry &q) {
    uint64_t slot = fastmod(q.key, a.B, a.Bm);
    for (uint32_t probe = 0; probe < kProbeLimit; ++probe) {
        const unsigned long long w0 = a.tab[slot].w0;
        if (w0 == q.key) {
            uint4 m = *reinterpret_cast<const uint4 *>(a.tab[slot].mbr);
            uint32_t cur[4] = {m.x, m.y, m.z, m.w};
            mbr_extend(a.tab[slot].mbr, q.x1, q.y1, q.x2, q.y2, cur);
            a.stamp[slot] = a.st;
            return false;
        }
        if (w0 == kEmptyKey) return true;
        slot = (slot + 1 == a.B) ? 0 : slot + 1;
    }
    atomicOr(&a.cnt->error_flags, GLINT_EF_TABLE_FULL);
    return false;
}

/* warp-collective: process queue entries [0, n) one per lane */
__device__ inline void drain_queue(const RefineArgs &a, QEntry *Q, uint32_t n) {
    const int lane = threadIdx.x & 31;
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t e = base + lane;
        bool isnew = false;
        QEntry q;
        if (e < n) {
            q = Q[e];
            isnew = table_touch(a, q);
        }
        const unsigned m = __ballot_sync(0xffffffffu, isnew);
        if (m) {
            unsigned long long off = 0;
            const int leader = __ffs(m) - 1;
            if (lane == leader) off = atomicAdd(&a.cnt->new_keys, (unsigned long long)__popc(m));
            off = __shfl_sync(0xffffffffu, off, leader);
            if (isnew) {
                const unsigned long long idx = off + __popc(m & ((1u << lane) - 1u));
                if (idx < a.new_cap) {
                    a.newlist[idx].key = q.key;
                    a.newlist[idx].prio = q.prio;
                } else {
                    atomicOr(&a.cnt->error_flags, GLINT_EF_NEW_OVERFLOW);
                }
            }
        }
    }
    __syncwarp();
}

/* warp-collective: append this lane's contact (if any) to the queue */
__device__ inline void enqueue(const RefineArgs &a, QEntry *Q, uint32_t &qn, bool hit, unsigned long long key,
                               unsigned long long prio, float x1, float y1, float x2, float y2) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (hit) {
        QEntry &e = Q[qn + __popc(m & ((1u << lane) - 1u))];
        e.key = key;
        e.prio = prio;
        e.x1 = x1;
        e.y1 = y1;
        e.x2 = x2;
        e.y2 = y2;
    }
    qn += __popc(m);
    __syncwarp();
    if (qn >= 32) {
        drain_queue(a, Q, 32);
        /* move the remainder to the front */
        const uint32_t rest = qn - 32;
        if ((uint32_t)lane < rest) Q[lane] = Q[32 + lane];
        __syncwarp();
        qn = rest;
    }
}

__device__ inline bool has_check(const RefineArgs &a, uint32_t obj, uint32_t gid) {
    const uint32_t b = a.qstart[obj], e = a.qstart[obj + 1];
    for (uint32_t k = b; k < e; ++k)
        if (a.qlist[k] == gid) return true;
    return false;
}

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
        for (uint32_t i = lane; i < k; i += 32) {
            const double2 p = a.sxy[s0 + i];
            sx[i] = p.x;
            sy[i] = p.y;
            sLm[i] = a.sL[s0 + i];
            sid[i] = a.sorted[s0 + i];
        }
        __syncwarp();
        /* inside checks: p1 = member i, p2 = member j > i (ids ascend with rank) */
        for (uint32_t i = 0; i + 1 < k; ++i) {
            const double x1 = sx[i], y1 = sy[i], L1 = sLm[i];
            const uint32_t p1 = sid[i];
            const float fx1 = (float)x1, fy1 = (float)y1;
            for (uint32_t jb = i + 1; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long key = 0;
                float fx2 = 0.f, fy2 = 0.f;
                if (j < k) {
                    ++cand;
                    const double x2 = sx[j], y2 = sy[j];
                    hit = point_le_exact(x1, y1, x2, y2, L1, a.ex);
                    if (hit) {
                        ++hits;
                        key = cantor(p1, sid[j]);
                        fx2 = (float)x2;
                        fy2 = (float)y2;
                    }
                }
                enqueue(a, Q, qn, hit, key, prio_pack(0, p1, 0, j), fx1, fy1, fx2, fy2);
            }
        }
        /* cross-leaf checks that target this leaf */
        const uint32_t tb = a.tstart[g], te = a.tstart[g + 1];
        for (uint32_t t = tb; t < te; ++t) {
            const uint2 qe = a.tlist[t];
            const uint32_t q = qe.x;
            const double2 qp = a.pts[q];
            const double Lq = a.L[q];
            const uint32_t qgid = a.obj_gid[q];
            const bool qstored = (a.rank_of[q] - a.grid_start[qgid]) < cap;
            const float fqx = (float)qp.x, fqy = (float)qp.y;
            for (uint32_t jb = 0; jb < k; jb += 32) {
                const uint32_t j = jb + lane;
                bool hit = false;
                unsigned long long key = 0;
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
                            key = q < m ? cantor(q, m) : cantor(m, q);
                            fx2 = (float)x2;
                            fy2 = (float)y2;
                        }
                    }
                }
                enqueue(a, Q, qn, hit, key, prio_pack(1, q, qe.y, j), fqx, fqy, fx2, fy2);
            }
        }
        __syncwarp();
    }
    drain_queue(a, Q, qn);
    /* warp totals */
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_down_sync(0xffffffffu, cand, o);
        hits += __shfl_down_sync(0xffffffffu, hits, o);
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->candidates, cand);
        atomicAdd(&a.cnt->contacts, hits);
    }
}

size_t refine_smem_bytes(uint32_t cap) {
    const size_t per_warp = (size_t)cap * 28 + sizeof(QEntry) * kQueue + 64;
    return (size_t)kRefineWarps * ((per_warp + 63) & ~(size_t)63);
}

cudaError_t launch_refine(glint_ctx *c, uint32_t /*cur_time*/) {
    RefineArgs a;
    a.work = c->d_leaf_work;
    a.grid_start = c->d_grid_start;
    a.grid_count = c->d_grid_count;
    a.sorted = c->d_sorted;
    a.sxy = c->d_sxy;
    a.sL = c->d_sL;
    a.tstart = c->d_tstart;
    a.tlist = c->d_tlist;
    a.pts = c->d_pts;
    a.L = c->d_L;
    a.obj_gid = c->d_obj_gid;
    a.rank_of = c->d_rank_of;
    a.qstart = c->d_qstart;
    a.qlist = c->d_qlist;
    a.tab = c->d_tab;
    a.stamp = c->d_stamp;
    a.newlist = c->d_new;
    a.B = c->B;
    a.Bm = c->Bm;
    a.new_cap = c->new_cap;
    a.cap = c->cap;
    a.st = stamp_of(c->step_index);
    a.ex = make_exact(c);
    a.cnt = c->d_cnt;
    const size_t smem = refine_smem_bytes(c->cap);
    k_refine_fp64<<<152 * 8, 32 * kRefineWarps, smem, c->stream>>>(a);
    return cudaGetLastError();
}

void refine_set_attributes(uint32_t cap) {
    cudaFuncSetAttribute(k_refine_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)refine_smem_bytes(cap));
}

/* ---- insertion of the step's new keys ------------------------------------
 * Deterministic linear probing with priority displacement: a key walking from
 * its home slot takes an empty slot, or swaps itself into a slot held by a
 * key inserted this step with a larger priority (which then walks on from the
 * next slot).  Committed keys are never moved.  The final layout is the one a
 * single thread produces by inserting the keys one by one in priority order,
 * which is the reference's order (tracing/refinement.cpp:34-55).  A key that
 * meets its own committed entry further along (left there when an earlier
 * slot of its probe run emptied) touches that entry instead, as the reference
 * does when its probe reaches it. */
__device__ inline bool u128_eq(const ulonglong2 &a, const ulonglong2 &b) { return a.x == b.x && a.y == b.y; }

/* a fresh read of a record's first 16 bytes (may be torn; every use is
 * validated by the compare-and-swap that follows) */
__device__ inline ulonglong2 ld_volatile_u128(const TRec *r) {
    ulonglong2 v;
    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(r));
    return v;
}

__device__ inline ulonglong2 cas128(TRec *r, ulonglong2 expect, ulonglong2 desired) {
    unsigned __int128 e = ((unsigned __int128)expect.y << 64) | expect.x;
    unsigned __int128 d = ((unsigned __int128)desired.y << 64) | desired.x;
    unsigned __int128 o = atomicCAS(reinterpret_cast<unsigned __int128 *>(r), e, d);
    return make_ulonglong2((unsigned long long)o, (unsigned long long)(o >> 64));
}

__global__ void __launch_bounds__(256) k_insert(const NewEntry *__restrict__ list, TRec *tab, uint8_t *stamp,
                                                uint64_t B, uint64_t Bm, uint64_t new_cap,
                                                const double2 *__restrict__ pts, uint8_t st, DevCounters *cnt) {
    const unsigned long long n0 = cnt->new_keys;
    const unsigned long long n = n0 < new_cap ? n0 : new_cap;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        ulonglong2 cur = make_ulonglong2(list[i].key | kNewFlag, list[i].prio);
        uint64_t slot = fastmod(list[i].key, B, Bm);
        bool done = false;
        for (uint32_t iter = 0; iter < kProbeLimit && !done; ++iter) {
            ulonglong2 seen = ld_volatile_u128(&tab[slot]);
            for (uint32_t retry = 0;; ++retry) {
                if (retry >= kProbeLimit) {
                    atomicOr(&cnt->error_flags, GLINT_EF_TABLE_FULL);
                    done = true;
                    break;
                }
                const unsigned long long plain = cur.x & kKeyMask;
                if (seen.x == kEmptyKey) {
                    ulonglong2 prev = cas128(&tab[slot], seen, cur);
                    if (u128_eq(prev, seen)) {
                        stamp[slot] = kStampNew;
                        done = true;
                        break;
                    }
                    seen = prev;
                    continue;
                }
                if (seen.x == plain) {
                    /* the carried key's own committed entry */
                    uint32_t pa, pb;
                    cantor_inverse(plain, pa, pb);
                    const double2 A = pts[pa], Bp = pts[pb];
                    uint4 m = *reinterpret_cast<const uint4 *>(tab[slot].mbr);
                    uint32_t curm[4] = {m.x, m.y, m.z, m.w};
                    mbr_extend(tab[slot].mbr, (float)A.x, (float)A.y, (float)Bp.x, (float)Bp.y, curm);
                    stamp[slot] = st;
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
                        cur = seen; /* the displaced key walks on */
                        break;
                    }
                    seen = prev;
                    continue;
                }
                break; /* occupied by a committed key or an earlier new key */
            }
            if (!done) slot = (slot + 1 == B) ? 0 : slot + 1;
        }
        if (!done) atomicOr(&cnt->error_flags, GLINT_EF_TABLE_FULL);
    }
}

cudaError_t launch_insert(glint_ctx *c, uint32_t /*cur_time*/) {
    k_insert<<<152 * 8, 256, 0, c->stream>>>(c->d_new, c->d_tab, c->d_stamp, c->B, c->Bm, c->new_cap, c->d_pts,
                                             stamp_of(c->step_index), c->d_cnt);
    return cudaGetLastError();
}

} // namespace glint
