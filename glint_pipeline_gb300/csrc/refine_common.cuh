/*
 * refine_common.cuh -- the contact queue shared by the refine kernels: pairs
 * within reach are compacted with a warp ballot into a per-warp shared
 * queue and applied to the meeting table 32 at a time.
 */
#ifndef GLINT_REFINE_COMMON_CUH_
#define GLINT_REFINE_COMMON_CUH_

#include "glint_internal.cuh"

namespace glint {

constexpr int kQueue = 96;      /* a drain of 64 plus one enqueue of up to 32 */
constexpr uint32_t kDrainAt = 64;
constexpr uint32_t kProbeLimit = 1u << 22;

struct QEntry {
    unsigned long long pw;     /* pair word (a << 32) | b, a < b */
    unsigned long long prio;   /* position in the reference's check order */
    float x1, y1, x2, y2;      /* the two points, rounded to f32 */
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
    const longlong2 *sipos;    /* fixed-point coordinates, leaf-major */
    const float2 *sfpos;       /* FP32 coordinates, leaf-major */
    const float *sc;           /* screening scale cx, leaf-major */
    const uint32_t *obj_gid;
    const uint32_t *rank_of;
    const uint32_t *qstart;
    const uint32_t *qlist;
    const uint2 *extra;        /* (leaf, chunk) items beyond each leaf's first chunk */
    TRec *tab;
    uint8_t *stamp;
    NewEntry *newlist;
    uint64_t B, Bm, new_cap;
    uint32_t cap;
    uint32_t chunk;            /* cross-leaf checks per work item */
    uint32_t extra_cap;        /* entries of `extra` */
    Frame f;
    ExactCtx ex;
    DevCounters *cnt;
};

/* The table as it stood at the start of the step: keys do not change while
 * the refine kernels run.  Found -> touch the entry (tag, f32 box; each pair
 * has at most one event per step, so the box needs no atomics).  Not found
 * before an empty slot -> the pair is new this step.  The walk starts at the
 * home slot, whose key word and box the caller has already loaded. */
__device__ inline bool table_touch_from(const RefineArgs &a, const QEntry &q, uint64_t slot, unsigned long long w0,
                                        uint4 m, uint32_t tag) {
    for (uint32_t probe = 0; probe < kProbeLimit; ++probe) {
        if (w0 == q.pw) {
            const uint32_t lx = min(fenc(q.x1), fenc(q.x2)), hx = max(fenc(q.x1), fenc(q.x2));
            const uint32_t ly = min(fenc(q.y1), fenc(q.y2)), hy = max(fenc(q.y1), fenc(q.y2));
            if (lx < m.x || ly < m.y || hx > m.z || hy > m.w) {
                m.x = min(m.x, lx);
                m.y = min(m.y, ly);
                m.z = max(m.z, hx);
                m.w = max(m.w, hy);
                *reinterpret_cast<uint4 *>(a.tab[slot].mbr) = m;
            }
            rec_set_tag(a.tab[slot], tag);
            return false;
        }
        if (w0 == kEmptyW0) return true;
        slot = (slot + 1 == a.B) ? 0 : slot + 1;
        w0 = a.tab[slot].w0;
        m = *reinterpret_cast<const uint4 *>(a.tab[slot].mbr);
    }
    atomicOr(&a.cnt->error_flags, GLINT_EF_TABLE_FULL);
    return false;
}

__device__ inline uint64_t home_slot(const RefineArgs &a, unsigned long long pw) {
    return fastmod(cantor(pair_a(pw), pair_b(pw)), a.B, a.Bm);
}

/* warp-collective: the lanes whose pair is new append it to the new list */
__device__ inline void append_new(const RefineArgs &a, bool isnew, const QEntry &q) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, isnew);
    if (!m) return;
    unsigned long long off = 0;
    const int leader = __ffs(m) - 1;
    if (lane == leader) off = atomicAdd(&a.cnt->new_keys, (unsigned long long)__popc(m));
    off = __shfl_sync(0xffffffffu, off, leader);
    if (isnew) {
        const unsigned long long idx = off + __popc(m & ((1u << lane) - 1u));
        if (idx < a.new_cap) {
            a.newlist[idx].key = q.pw;
            a.newlist[idx].prio = q.prio;
        } else {
            atomicOr(&a.cnt->error_flags, GLINT_EF_NEW_OVERFLOW);
        }
    }
}

/* warp-collective: process queue entries [0, n), two per lane, with both
 * home records requested before either is used (the table is far larger
 * than L2, so each is a DRAM round trip) */
__device__ inline void drain_queue(const RefineArgs &a, QEntry *Q, uint32_t n, uint32_t tag) {
    const int lane = threadIdx.x & 31;
    for (uint32_t base = 0; base < n; base += 64) {
        const uint32_t e0 = base + lane, e1 = base + 32 + lane;
        const bool v0 = e0 < n, v1 = e1 < n;
        QEntry q0, q1;
        uint64_t s0 = 0, s1 = 0;
        if (v0) {
            q0 = Q[e0];
            s0 = home_slot(a, q0.pw);
        }
        if (v1) {
            q1 = Q[e1];
            s1 = home_slot(a, q1.pw);
        }
        /* out-of-range lanes read slot 0, which exists, and ignore it */
        const unsigned long long w00 = a.tab[s0].w0, w01 = a.tab[s1].w0;
        const uint4 m0 = *reinterpret_cast<const uint4 *>(a.tab[s0].mbr);
        const uint4 m1 = *reinterpret_cast<const uint4 *>(a.tab[s1].mbr);
        const bool n0 = v0 && table_touch_from(a, q0, s0, w00, m0, tag);
        const bool n1 = v1 && table_touch_from(a, q1, s1, w01, m1, tag);
        append_new(a, n0, q0);
        append_new(a, n1, q1);
    }
    __syncwarp();
}

/* warp-collective: append this lane's contact (if any) to the queue */
__device__ inline void enqueue(const RefineArgs &a, QEntry *Q, uint32_t &qn, bool hit, unsigned long long pw,
                               unsigned long long prio, float x1, float y1, float x2, float y2, uint32_t tag) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (hit) {
        QEntry &e = Q[qn + __popc(m & ((1u << lane) - 1u))];
        e.pw = pw;
        e.prio = prio;
        e.x1 = x1;
        e.y1 = y1;
        e.x2 = x2;
        e.y2 = y2;
    }
    qn += __popc(m);
    __syncwarp();
    if (qn >= kDrainAt) {
        drain_queue(a, Q, kDrainAt, tag);
        const uint32_t rest = qn - kDrainAt;
        if ((uint32_t)lane < rest) Q[lane] = Q[kDrainAt + lane];
        __syncwarp();
        qn = rest;
    }
}

/* Work items: a leaf's inside pairs with its first `chunk` cross-leaf
 * checks, and one item per further chunk of its checks.  Dense leaves are
 * the target of thousands of checks; split into chunks they spread over the
 * warps instead of leaving a long tail on one.  Every event carries its
 * position in the reference's order, so the split does not change results. */
/* warp-collective: the next item, extra chunks first (the long work first);
 * false when none is left */
__device__ inline bool claim_item(const RefineArgs &a, uint32_t nwork, uint32_t n_extra, bool &extra_done,
                                  uint32_t &g, uint32_t &chunk) {
    const int lane = threadIdx.x & 31;
    uint32_t v = 0, kind = 0;
    if (lane == 0) {
        if (!extra_done) {
            v = atomicAdd(&a.cnt->extra_next, 1u);
            if (v < n_extra && v < a.extra_cap) kind = 1;
        }
        if (kind == 0) {
            v = atomicAdd(&a.cnt->work_next, 1u);
            kind = v < nwork ? 2u : 0u;
        }
    }
    kind = __shfl_sync(0xffffffffu, kind, 0);
    v = __shfl_sync(0xffffffffu, v, 0);
    if (kind == 1) {
        const uint2 e = a.extra[v];
        g = e.x;
        chunk = e.y;
        return true;
    }
    extra_done = true;
    if (kind == 2) {
        g = a.work[v];
        chunk = 0;
        return true;
    }
    return false;
}

/* the cross-leaf checks of one item */
__device__ inline void item_checks(const RefineArgs &a, uint32_t g, uint32_t chunk, uint32_t &tb, uint32_t &te) {
    const uint32_t b = a.tstart[g], e = a.tstart[g + 1];
    tb = b + chunk * a.chunk;
    te = tb + a.chunk < e ? tb + a.chunk : e;
    if (tb > e) tb = e;
}

/* does object obj have a cross-leaf check on grid gid */
__device__ inline bool has_check(const RefineArgs &a, uint32_t obj, uint32_t gid) {
    const uint32_t b = a.qstart[obj], e = a.qstart[obj + 1];
    for (uint32_t k = b; k < e; ++k)
        if (a.qlist[k] == gid) return true;
    return false;
}

__device__ inline unsigned long long pw_of(uint32_t p, uint32_t q) { return p < q ? pair_word(p, q) : pair_word(q, p); }

} // namespace glint

#endif
