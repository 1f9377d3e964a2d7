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

/* lookup_rec from node `start`; calls emit(gid, ordinal) in walk order;
 * returns the number of leaves kept */
template <class Emit>
__device__ inline uint32_t lookup_walk(const DNode *__restrict__ nodes, const double2 *__restrict__ low, uint32_t start,
                                       double px, double py, double Lp, const FastBox &fb, const ExactCtx &ex, DevCounters *cnt,
                                       Emit emit) {
    uint32_t st_node[kStackMax];
    uint8_t st_next[kStackMax];
    int sp = 0;
    st_node[0] = start;
    st_next[0] = 0;
    sp = 1;
    uint32_t kept = 0;
    const float iLf = (float)(1.0 / Lp);
    while (sp > 0) {
        const int top = sp - 1;
        const uint8_t i = st_next[top];
        if (i == 4) { --sp; continue; }
        st_next[top] = i + 1;
        const uint32_t ch = nodes[st_node[top]].child[i];
        const DNode n = nodes[ch];
        const double2 lo = low[ch];
        if (box_le_fast(lo.x, lo.y, n.high_x, n.high_y, px, py, Lp, iLf, fb, ex)) {
            if (n.type == kLeaf) {
                if (py < lo.y || (py < n.high_y && px < lo.x)) {
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

__global__ void __launch_bounds__(128) k_filter_walk(const uint32_t *__restrict__ sorted, uint32_t N,
                                                     const double2 *__restrict__ pts, const double *__restrict__ L,
                                                     const uint32_t *__restrict__ obj_lv,
                                                     const uint32_t *__restrict__ obj_leaf,
                                                     const DNode *__restrict__ nodes, const double2 *__restrict__ low,
                                                     uint32_t *__restrict__ qcount, uint32_t *__restrict__ qtmp,
                                                     FastBox fb, ExactCtx ex, DevCounters *cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const uint32_t pid = sorted[i];
        const uint32_t lv = obj_lv[pid];
        uint32_t kept = 0;
        if (lv != obj_leaf[pid]) {
            const double2 p = pts[pid];
            uint32_t *row = qtmp + (size_t)pid * kQInline;
            kept = lookup_walk(nodes, low, lv, p.x, p.y, L[pid], fb, ex, cnt, [&](uint32_t gid, uint32_t k) {
                if (k < kQInline) row[k] = gid;
            });
            atomicAdd(&cnt->border_objects, 1u);
        }
        qcount[pid] = kept;
    }
}

__global__ void __launch_bounds__(128) k_filter_emit(uint32_t N, const double2 *__restrict__ pts,
                                                     const double *__restrict__ L, const uint32_t *__restrict__ obj_lv,
                                                     const DNode *__restrict__ nodes, const double2 *__restrict__ low,
                                                     const uint32_t *__restrict__ qstart,
                                                     const uint32_t *__restrict__ qtmp, uint32_t *__restrict__ qlist,
                                                     uint32_t *__restrict__ tcount, uint64_t check_cap, FastBox fb, ExactCtx ex,
                                                     DevCounters *cnt) {
    for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < N; pid += gridDim.x * blockDim.x) {
        const uint32_t b = qstart[pid], e = qstart[pid + 1];
        if (b == e) continue;
        if ((uint64_t)e > check_cap) {
            atomicOr(&cnt->error_flags, GLINT_EF_CHECKS_OVERFLOW);
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
            const double2 p = pts[pid];
            lookup_walk(nodes, low, obj_lv[pid], p.x, p.y, L[pid], fb, ex, cnt, [&](uint32_t gid, uint32_t k) {
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
    ExactCtx ex = make_exact(c);
    FastBox fb;
    const double r2 = c->cfg.reach_distance * c->cfg.reach_distance;
    fb.iMf = (float)(1.0 / c->dpm_lat);
    fb.r2lo = (float)(r2 * (1.0 - std::ldexp(1.0, -16)));
    fb.r2hi = (float)(r2 * (1.0 + std::ldexp(1.0, -16)));
    k_filter_walk<<<grid_for(N, 128, 152u * 16u), 128, 0, s>>>(c->d_sorted, N, c->d_pts, c->d_L, c->d_obj_lv,
                                                                 c->d_obj_leaf, c->d_nodes, c->d_low, c->d_qcount,
                                                                 c->d_qtmp, fb, ex, c->d_cnt);
    scan_u32(c->d_qcount, c->d_qstart, N, c->d_scan_tmp, s);
    cudaMemsetAsync(c->d_tcount, 0, sizeof(uint32_t) * (G + 1), s);
    cudaMemsetAsync(c->d_tcursor, 0, sizeof(uint32_t) * G, s);
    k_filter_emit<<<grid_for(N, 128, 152u * 16u), 128, 0, s>>>(N, c->d_pts, c->d_L, c->d_obj_lv, c->d_nodes, c->d_low,
                                                                 c->d_qstart, c->d_qtmp,
                                                                 c->d_qlist, c->d_tcount, c->check_cap, fb, ex, c->d_cnt);
    scan_u32(c->d_tcount, c->d_tstart, G, c->d_scan_tmp, s);
    k_filter_group<<<grid_for(N, 256, 152u * 8u), 256, 0, s>>>(N, c->d_qstart, c->d_qlist, c->d_tstart, c->d_tcursor,
                                                                c->d_tlist, c->check_cap);
    return cudaGetLastError();
}

} // namespace glint
