/*
 * k_partition.cu -- stage (a): assign every object to its quadtree leaf and
 * lay the objects out leaf-major.
 *
 * Reference: the phased descent of filter_unit (tracing/filter.cpp:228-245)
 * and cuda_partition (cuda/geometry.cu:221-271): child = (y>mid_y)*2 +
 * (x>mid_x) from the root until a leaf, tracking last_valid, the deepest node
 * on the path whose top and right edges are more than x_buffer/y_buffer away.
 * workbench::insert (tracing/filter.cpp:95-111) then appends the object to
 * its leaf buffer and drops it once the buffer holds grid_capacity*amplify
 * objects; with one thread objects arrive in id order, so a leaf's stored
 * members are its smallest ids.
 *
 * Here the leaf buffers are replaced by a stable sort of objects by
 * (grid id, object id): a count per grid, an exclusive scan, a scatter and a
 * per-leaf sort of each segment.  The first min(count, capacity) entries of a
 * segment are exactly the reference's stored members, in the same order.
 */
#include "glint_internal.cuh"

namespace glint {

constexpr int kMaxDepth = 64;

__global__ void __launch_bounds__(256) k_descend(const double2 *__restrict__ pts, const uint32_t *__restrict__ order,
                                                 uint32_t N, const DNode *__restrict__ nodes, uint32_t S, uint32_t G,
                                                 double xb, double yb,
                                                 uint32_t *__restrict__ obj_gid, uint32_t *__restrict__ obj_lv,
                                                 uint32_t *__restrict__ obj_leaf, uint32_t *__restrict__ grid_count,
                                                 DevCounters *cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const uint32_t pid = order[i];
        const double2 p = pts[pid];
        /* the comparisons of filter.cpp:231,235-236 on order-preserving keys */
        const uint64_t kx = dkey(p.x), ky = dkey(p.y);
        const uint64_t kxb = dkey(__dadd_rn(p.x, xb)), kyb = dkey(__dadd_rn(p.y, yb));
        uint32_t cur = 0, lv = 0, gid = 0;
        DNode n = nodes[0];
        int depth = 0;
        for (;;) {
            const int child = (ky > n.kmy) * 2 + (kx > n.kmx);
            cur = n.child[child];
            if (cur >= S || ++depth >= kMaxDepth) {
                /* a corrupt or too deep schema: keep memory safe and report */
                atomicOr(&cnt->error_flags, GLINT_EF_TREE_DEPTH);
                cur = lv = gid = 0;
                break;
            }
            n = nodes[cur];
            if (kxb < n.khx && kyb < n.khy) lv = cur;
            if (n.type == kLeaf) {
                gid = n.gid < G ? n.gid : 0u;
                break;
            }
            if (n.type != kBranch) {
                atomicOr(&cnt->error_flags, GLINT_EF_TREE_DEPTH);
                cur = lv = gid = 0;
                break;
            }
        }
        obj_gid[pid] = gid;
        obj_lv[pid] = lv;
        obj_leaf[pid] = cur;
        /* objects come in the previous step's leaf order, so the lanes of a
         * warp mostly share a leaf: one atomic per leaf and warp */
        const unsigned peers = __match_any_sync(__activemask(), gid);
        if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&grid_count[gid], (uint32_t)__popc(peers));
    }
}

__global__ void __launch_bounds__(256) k_scatter(const uint32_t *__restrict__ obj_gid, uint32_t N,
                                                 const uint32_t *__restrict__ grid_start,
                                                 uint32_t *__restrict__ grid_cursor, uint32_t *__restrict__ sorted) {
    for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < N; pid += gridDim.x * blockDim.x) {
        uint32_t g = obj_gid[pid];
        uint32_t pos = grid_start[g] + atomicAdd(&grid_cursor[g], 1u);
        sorted[pos] = pid;
    }
}

/* leaves that hold objects, and the objects their buffers drop */
__global__ void __launch_bounds__(256) k_leaf_work(const uint32_t *__restrict__ grid_count, uint32_t G, uint32_t cap,
                                                   uint32_t *__restrict__ work, uint32_t *__restrict__ big,
                                                   uint32_t warp_limit, DevCounters *cnt) {
    const int lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x; base < G; base += gridDim.x * blockDim.x) {
        uint32_t g = base + threadIdx.x;
        uint32_t c = g < G ? grid_count[g] : 0u;
        bool has = c > 0;
        unsigned m = __ballot_sync(0xffffffffu, has);
        uint32_t off = 0;
        if (lane == 0 && m) off = atomicAdd(&cnt->n_leaf_work, (unsigned)__popc(m));
        off = __shfl_sync(0xffffffffu, off, 0);
        if (has) work[off + __popc(m & ((1u << lane) - 1u))] = g;
        uint32_t drop = c > cap ? c - cap : 0u;
        for (int o = 16; o > 0; o >>= 1) drop += __shfl_down_sync(0xffffffffu, drop, o);
        if (lane == 0 && drop) atomicAdd(&cnt->dropped, drop);
        /* segments too long for one warp go to the block sorter */
        bool isbig = c > warp_limit;
        unsigned mb = __ballot_sync(0xffffffffu, isbig);
        uint32_t boff = 0;
        if (lane == 0 && mb) boff = atomicAdd(&cnt->n_big, (unsigned)__popc(mb));
        boff = __shfl_sync(0xffffffffu, boff, 0);
        if (isbig) big[boff + __popc(mb & ((1u << lane) - 1u))] = g;
    }
}

/* bitonic sort of n (<= 1024) keys in a warp's shared buffer, padded with ~0u */
__device__ inline void warp_bitonic(uint32_t *buf, uint32_t n) {
    uint32_t P = 32;
    while (P < n) P <<= 1;
    const int lane = threadIdx.x & 31;
    for (uint32_t i = n + lane; i < P; i += 32) buf[i] = 0xffffffffu;
    __syncwarp();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < P; i += 32) {
                uint32_t l = i ^ j;
                if (l > i) {
                    uint32_t a = buf[i], b = buf[l];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) { buf[i] = b; buf[l] = a; }
                }
            }
            __syncwarp();
        }
    }
}

constexpr int kSortWarps = 8;
constexpr uint32_t kWarpSortMax = 1024;

/* one warp per leaf segment of up to kWarpSortMax objects */
__global__ void __launch_bounds__(32 * kSortWarps) k_segsort_warp(const uint32_t *__restrict__ work,
                                                                  const uint32_t *__restrict__ grid_start,
                                                                  const uint32_t *__restrict__ grid_count,
                                                                  uint32_t *__restrict__ sorted, const DevCounters *cnt) {
    __shared__ uint32_t buf[kSortWarps][kWarpSortMax];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nwork = cnt->n_leaf_work;
    for (uint32_t li = blockIdx.x * kSortWarps + w; li < nwork; li += gridDim.x * kSortWarps) {
        const uint32_t g = work[li];
        const uint32_t n = grid_count[g];
        if (n <= 1 || n > kWarpSortMax) continue;
        uint32_t *seg = sorted + grid_start[g];
        if (n <= 32) {
            uint32_t v = lane < (int)n ? seg[lane] : 0xffffffffu;
            /* register bitonic sort across the warp */
            for (int k = 2; k <= 32; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    uint32_t o = __shfl_xor_sync(0xffffffffu, v, j);
                    bool up = (lane & k) == 0;
                    bool lower = (lane & j) == 0;
                    v = (lower == up) ? min(v, o) : max(v, o);
                }
            }
            if (lane < (int)n) seg[lane] = v;
        } else {
            for (uint32_t i = lane; i < n; i += 32) buf[w][i] = seg[i];
            __syncwarp();
            warp_bitonic(buf[w], n);
            for (uint32_t i = lane; i < n; i += 32) seg[i] = buf[w][i];
        }
        __syncwarp();
    }
}

constexpr uint32_t kBlockSortMax = 16384;

/* one block per long segment (up to kBlockSortMax objects) */
__global__ void __launch_bounds__(1024) k_segsort_block(const uint32_t *__restrict__ big,
                                                        const uint32_t *__restrict__ grid_start,
                                                        const uint32_t *__restrict__ grid_count,
                                                        uint32_t *__restrict__ sorted, DevCounters *cnt) {
    extern __shared__ uint32_t sbuf[];
    const uint32_t nbig = cnt->n_big;
    for (uint32_t bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
        const uint32_t g = big[bi];
        const uint32_t n = grid_count[g];
        if (n > kBlockSortMax) {
            if (threadIdx.x == 0) atomicOr(&cnt->error_flags, GLINT_EF_SEGMENT_TOO_LARGE);
            continue;
        }
        uint32_t P = 1024;
        while (P < n) P <<= 1;
        uint32_t *seg = sorted + grid_start[g];
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) sbuf[i] = i < n ? seg[i] : 0xffffffffu;
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                    uint32_t l = i ^ j;
                    if (l > i) {
                        uint32_t a = sbuf[i], b = sbuf[l];
                        bool up = (i & k) == 0;
                        if ((a > b) == up) { sbuf[i] = b; sbuf[l] = a; }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) seg[i] = sbuf[i];
        __syncthreads();
    }
}

/* per object, in leaf-major order: the coordinates, their fixed-point and
 * FP32 forms and the screening scale cx; L with CUDA sin for the plain form;
 * each object's sorted position */
struct GatherOut {
    double2 *sxy;
    longlong2 *sipos;
    float2 *sfpos;
    float *sc;
    double *sL;        /* null: not needed */
    float2 *fpos;      /* by object id */
    uint32_t *rank_of;
};

__global__ void __launch_bounds__(256) k_gather(const uint32_t *__restrict__ sorted, uint32_t N,
                                                const double2 *__restrict__ pts, GatherOut o, Frame f) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const uint32_t pid = sorted[i];
        const double2 p = pts[pid];
        o.sxy[i] = p;
        bool clamped = false;
        const long long X = fx_coord(p.x, f.ox, f.S, &clamped);
        const long long Y = fx_coord(p.y, f.oy, f.S, &clamped);
        o.sipos[i] = make_longlong2(X, Y);
        o.sc[i] = clamped ? __int_as_float(0x7fc00000) : c_of_lat(p.y, f);
        const float2 fp = make_float2((float)p.x, (float)p.y);
        o.sfpos[i] = fp;
        o.fpos[pid] = fp;
        if (o.sL) o.sL[i] = dpm_lon_fast(p.y);
        o.rank_of[pid] = i;
    }
}

cudaError_t launch_partition(glint_ctx *c, uint32_t /*cur_time*/) {
    cudaStream_t s = c->stream;
    const uint32_t N = c->N, G = c->G;
    cudaMemsetAsync(c->d_grid_count, 0, sizeof(uint32_t) * (G + 1), s);
    cudaMemsetAsync(c->d_grid_cursor, 0, sizeof(uint32_t) * G, s);
    k_descend<<<grid_for(N, 256, 152u * 8u), 256, 0, s>>>(c->d_pts, c->d_order, N, c->d_nodes, c->S, G, c->x_buffer,
                                                           c->y_buffer, c->d_obj_gid, c->d_obj_lv, c->d_obj_leaf,
                                                           c->d_grid_count, c->d_cnt);
    scan_u32(c->d_grid_count, c->d_grid_start, G, c->d_scan_tmp, s);
    k_scatter<<<grid_for(N, 256, 152u * 8u), 256, 0, s>>>(c->d_obj_gid, N, c->d_grid_start, c->d_grid_cursor,
                                                           c->d_sorted);
    k_leaf_work<<<grid_for(G, 256, 152u * 8u), 256, 0, s>>>(c->d_grid_count, G, c->cap, c->d_leaf_work, c->d_big,
                                                             kWarpSortMax, c->d_cnt);
    k_segsort_warp<<<152 * 8, 32 * kSortWarps, 0, s>>>(c->d_leaf_work, c->d_grid_start, c->d_grid_count, c->d_sorted,
                                                       c->d_cnt);
    k_segsort_block<<<152, 1024, kBlockSortMax * sizeof(uint32_t), s>>>(c->d_big, c->d_grid_start, c->d_grid_count,
                                                                        c->d_sorted, c->d_cnt);
    GatherOut o;
    o.sxy = c->d_sxy;
    o.sipos = c->d_sipos;
    o.sfpos = c->d_sfpos;
    o.sc = c->d_sc;
    o.sL = c->cfg.precision_mode == 1 ? nullptr : c->d_sL;
    o.fpos = c->d_fpos;
    o.rank_of = c->d_rank_of;
    k_gather<<<grid_for(N, 256, 152u * 8u), 256, 0, s>>>(c->d_sorted, N, c->d_pts, o, c->frame);
    /* this step's leaf-major order is the next descent's processing order */
    cudaMemcpyAsync(c->d_order, c->d_sorted, sizeof(uint32_t) * N, cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError();
}

void partition_set_attributes() {
    cudaFuncSetAttribute(k_segsort_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kBlockSortMax * sizeof(uint32_t)));
}

} // namespace glint
