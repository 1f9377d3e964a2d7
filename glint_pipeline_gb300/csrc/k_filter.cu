/*
 * k_filter.cu -- stage (b) part 1: cross-leaf checks for objects near the top
 * or right border of their leaf.
 *
 * Reference: filter_unit (tracing/filter.cpp:247-261) runs lookup_rec
 * (tracing/filter.cpp:130-152) from last_valid for every object whose
 * last_valid is not its own leaf: a depth-first walk over children 0..3 that
 * descends into branches within reach (box::distance, geometry/geometry.h:
 * 174-185) and keeps a leaf when it is within reach and lies above the
 * object, or level with and to its right.  Each kept leaf becomes a check
 * (object, leaf grid id, inside = false) appended after the N inside checks,
 * in object order and, per object, in walk order.
 *
 * Device form: one thread per border object, objects visited in leaf-major
 * order so that neighbouring threads walk the same nodes.  The walk is done
 * once; up to kQInline targets per object are kept in a scratch row, and the
 * rare object with more re-walks in the second pass.  The checks are stored
 * twice: by querier (CSR over object ids, for the duplicate rule in refine)
 * and grouped by target leaf (for the refine tiles).
 */
#include <cmath>

#include "glint_internal.cuh"

namespace glint {

constexpr int kQInline = 8;
constexpr int kStackMax = 64;

/* the querier of a walk: exact coordinates (for the top/right rule and the
 * exact fallback), fixed-point coordinates and screening limits */
struct WalkPoint {
    double px, py;
    uint64_t kx, ky;     /* dkey(px), dkey(py) */
    long long X, Y;
    Screen sc;
};

__device__ inline WalkPoint walk_point(const double2 p, const longlong2 ip, float c, const Frame &f) {
    WalkPoint w;
    w.px = p.x;
    w.py = p.y;
    w.kx = dkey(p.x);
    w.ky = dkey(p.y);
    w.X = ip.x;
    w.Y = ip.y;
    w.sc = make_screen(c, f);
    return w;
}

/* the reference's FP64 box test for a box inside the guard band (rare); kept
 * out of line so that none of its FP64 work is scheduled on the common path */
__device__ __noinline__ bool box_exact(double lx, double ly, double hx, double hy, double px, double py,
                                       const ExactCtx &ex) {
    return box_le_exact(lx, ly, hx, hy, px, py, dpm_lon_fast(py), ex);
}

/* lookup_rec from node `start`; calls emit(gid, ordinal) in walk order;
 * returns the number of leaves kept.  The box test is screened on the
 * fixed-point boxes; only a box within the guard band of the reach takes the
 * reference's FP64 box distance. */
template <class Emit>
__device__ inline uint32_t lookup_walk(const DNode *__restrict__ nodes, const double2 *__restrict__ low,
                                       const IBox *__restrict__ ibox, uint32_t start, const WalkPoint &w,
                                       const Frame &f, const ExactCtx &ex, DevCounters *cnt, Emit emit) {
    uint32_t st_node[kStackMax];
    uint8_t st_next[kStackMax];
    int sp = 0;
    st_node[0] = start;
    st_next[0] = 0;
    sp = 1;
    uint32_t kept = 0;
    while (sp > 0) {
        const int top = sp - 1;
        const uint8_t i = st_next[top];
        if (i == 4) { --sp; continue; }
        st_next[top] = i + 1;
        const uint32_t ch = nodes[st_node[top]].child[i];
        const DNode n = nodes[ch];
        int in = fx_box_screen(ibox[ch], w.X, w.Y, w.sc, f.cy);
        double2 lo;
        bool have_lo = false;
        if (in < 0) {
            atomicAdd(&cnt->box_band, 1u);
            lo = low[ch];
            have_lo = true;
            in = box_exact(lo.x, lo.y, kdbl(n.khx), kdbl(n.khy), w.px, w.py, ex) ? 1 : 0;
        }
        if (in) {
            if (n.type == kLeaf) {
                if (!have_lo) lo = low[ch];
                const uint64_t kly = dkey(lo.y), klx = dkey(lo.x);
                if (w.ky < kly || (w.ky < n.khy && w.kx < klx)) {
                    emit(n.gid, kept);
                    ++kept;
                }
            } else if (n.type == kBranch && sp < kStackMax) {
                st_node[sp] = ch;
                st_next[sp] = 0;
                ++sp;
            } else {
                atomicOr(&cnt->error_flags, GLINT_EF_DFS_OVERFLOW);
            }
        }
    }
    return kept;
}

struct FilterArgs {
    const uint32_t *sorted;
    const uint32_t *rank_of;
    const double2 *sxy;
    const longlong2 *sipos;
    const float *sc;
    const uint32_t *obj_lv;
    const uint32_t *obj_leaf;
    const DNode *nodes;
    const double2 *low;
    const IBox *ibox;
    uint32_t N;
    Frame f;
    ExactCtx ex;
    DevCounters *cnt;
};

/* Only border objects (a leaf beside their own in reach) walk the tree:
 * about half of them at 10M objects.  Each warp reads 32 consecutive ranks
 * at a time, queues its border objects in shared memory, and walks them 32 at
 * a time, so that every lane of a walk has an object. */
constexpr int kWalkWarps = 4;

__global__ void __launch_bounds__(32 * kWalkWarps) k_filter_walk(FilterArgs a, uint32_t *__restrict__ qcount,
                                                                 uint32_t *__restrict__ qtmp) {
    __shared__ uint32_t sbuf[kWalkWarps][64];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t stride = gridDim.x * kWalkWarps * 32;
    uint32_t nb = 0, nborder = 0;
    for (uint32_t base = (blockIdx.x * kWalkWarps + wid) * 32;; base += stride) {
        const bool more = base < a.N;
        if (more) {
            const uint32_t i = base + lane;
            bool border = false;
            if (i < a.N) {
                const uint32_t pid = a.sorted[i];
                border = a.obj_lv[pid] != a.obj_leaf[pid];
                if (!border) qcount[pid] = 0;
            }
            const unsigned m = __ballot_sync(0xffffffffu, border);
            if (border) sbuf[wid][nb + __popc(m & ((1u << lane) - 1u))] = i;
            nb += __popc(m);
            nborder += __popc(m);
            __syncwarp();
        }
        if (nb >= 32 || (!more && nb > 0)) {
            const uint32_t take = nb < 32 ? nb : 32;
            if ((uint32_t)lane < take) {
                const uint32_t i = sbuf[wid][lane];
                const uint32_t pid = a.sorted[i];
                const WalkPoint w = walk_point(a.sxy[i], a.sipos[i], a.sc[i], a.f);
                uint32_t *row = qtmp + (size_t)pid * kQInline;
                qcount[pid] = lookup_walk(a.nodes, a.low, a.ibox, a.obj_lv[pid], w, a.f, a.ex, a.cnt,
                                          [&](uint32_t gid, uint32_t k) {
                                              if (k < kQInline) row[k] = gid;
                                          });
            }
            const uint32_t rest = nb - take;
            __syncwarp();
            const uint32_t v = (uint32_t)lane < rest ? sbuf[wid][32 + lane] : 0u;
            __syncwarp();
            if ((uint32_t)lane < rest) sbuf[wid][lane] = v;
            __syncwarp();
            nb = rest;
        }
        if (!more && nb == 0) break;
    }
    if (lane == 0 && nborder) atomicAdd(&a.cnt->border_objects, nborder);
}

__global__ void __launch_bounds__(128) k_filter_emit(FilterArgs a, const uint32_t *__restrict__ qstart,
                                                     const uint32_t *__restrict__ qtmp, uint32_t *__restrict__ qlist,
                                                     uint32_t *__restrict__ tcount, uint64_t check_cap) {
    for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < a.N; pid += gridDim.x * blockDim.x) {
        const uint32_t b = qstart[pid], e = qstart[pid + 1];
        if (b == e) continue;
        if ((uint64_t)e > check_cap) {
            atomicOr(&a.cnt->error_flags, GLINT_EF_CHECKS_OVERFLOW);
            continue;
        }
        const uint32_t n = e - b;
        const uint32_t *row = qtmp + (size_t)pid * kQInline;
        for (uint32_t k = 0; k < n && k < (uint32_t)kQInline; ++k) {
            uint32_t g = row[k];
            qlist[b + k] = g;
            atomicAdd(&tcount[g], 1u);
        }
        if (n > (uint32_t)kQInline) {
            const uint32_t r = a.rank_of[pid];
            const WalkPoint w = walk_point(a.sxy[r], a.sipos[r], a.sc[r], a.f);
            lookup_walk(a.nodes, a.low, a.ibox, a.obj_lv[pid], w, a.f, a.ex, a.cnt, [&](uint32_t gid, uint32_t k) {
                if (k >= (uint32_t)kQInline && k < n) {
                    qlist[b + k] = gid;
                    atomicAdd(&tcount[gid], 1u);
                }
            });
        }
    }
}

/* group the checks by target leaf: tlist entries are (querier, ordinal) */
__global__ void __launch_bounds__(256) k_filter_group(uint32_t N, const uint32_t *__restrict__ qstart,
                                                      const uint32_t *__restrict__ qlist,
                                                      const uint32_t *__restrict__ tstart,
                                                      uint32_t *__restrict__ tcursor, uint2 *__restrict__ tlist,
                                                      uint64_t check_cap) {
    for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < N; pid += gridDim.x * blockDim.x) {
        const uint32_t b = qstart[pid], e = qstart[pid + 1];
        if (b == e || (uint64_t)e > check_cap) continue;
        for (uint32_t k = b; k < e; ++k) {
            uint32_t g = qlist[k];
            uint32_t pos = tstart[g] + atomicAdd(&tcursor[g], 1u);
            tlist[pos] = make_uint2(pid, k - b);
        }
    }
}

cudaError_t launch_filter(glint_ctx *c) {
    cudaStream_t s = c->stream;
    const uint32_t N = c->N, G = c->G;
    FilterArgs a;
    a.sorted = c->d_sorted;
    a.rank_of = c->d_rank_of;
    a.sxy = c->d_sxy;
    a.sipos = c->d_sipos;
    a.sc = c->d_sc;
    a.obj_lv = c->d_obj_lv;
    a.obj_leaf = c->d_obj_leaf;
    a.nodes = c->d_nodes;
    a.low = c->d_low;
    a.ibox = c->d_ibox;
    a.N = N;
    a.f = c->frame;
    a.ex = make_exact(c);
    a.cnt = c->d_cnt;
    k_filter_walk<<<grid_for(N, 32 * kWalkWarps, 152u * 16u), 32 * kWalkWarps, 0, s>>>(a, c->d_qcount, c->d_qtmp);
    scan_u32(c->d_qcount, c->d_qstart, N, c->d_scan_tmp, s);
    cudaMemsetAsync(c->d_tcount, 0, sizeof(uint32_t) * (G + 1), s);
    cudaMemsetAsync(c->d_tcursor, 0, sizeof(uint32_t) * G, s);
    k_filter_emit<<<grid_for(N, 128, 152u * 16u), 128, 0, s>>>(a, c->d_qstart, c->d_qtmp, c->d_qlist, c->d_tcount,
                                                                 c->check_cap);
    scan_u32(c->d_tcount, c->d_tstart, G, c->d_scan_tmp, s);
    k_filter_group<<<grid_for(N, 256, 152u * 8u), 256, 0, s>>>(N, c->d_qstart, c->d_qlist, c->d_tstart, c->d_tcursor,
                                                                c->d_tlist, c->check_cap);
    return cudaGetLastError();
}

} // namespace glint
