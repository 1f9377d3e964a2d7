/*
 * k_schema.cu -- stage (a) part 2: split over-full leaves and merge
 * under-full quads, with the reference's one-step delay.
 *
 * Reference: update_schema_unit (tracing/filter.cpp:377-424) visits every
 * schema slot in index order.  A LEAF with width(true) > 2*reach and more than
 * grid_capacity objects counts an overflow and is split (split_node,
 * :338-375) once the count reaches schema_update_delay.  A BRANCH whose four
 * children are leaves holding fewer than grid_capacity objects together counts
 * an underflow and is merged (merge_node, :316-336).  Split pops four schema
 * slots and (after pushing the parent's grid) four grid ids from two stacks;
 * merge pushes the children back.  Because the pass runs in slot order, a
 * merge can make its parent's children all leaves before the parent is
 * visited (a cascade), and the slots and grid ids a split receives depend on
 * every earlier split and merge of the pass.
 *
 * Device form, same result:
 *  1. k_sch_collect: per slot, the split decision of each leaf and the merge
 *     decision of each branch whose children are all leaves; branches whose
 *     branch children all have smaller slots are merge candidates.
 *  2. k_sch_cascade: one block resolves the candidates bottom-up.
 *  3. events (split or merge) compacted in slot order.
 *  4. k_sch_stacks: one block replays the stack pushes and pops in event order
 *     inside a shared-memory window of both stacks, one thread doing the
 *     index arithmetic over event data staged by the whole block.
 *  5. k_sch_apply_merge then k_sch_apply_split write the node records.
 */
#include "glint_internal.cuh"

namespace glint {

enum : uint8_t { kEvNone = 0, kEvSplit = 1, kEvMerge = 2, kEvCand = 3, kEvFreed = 4 };

__global__ void __launch_bounds__(256) k_sch_collect(DNode *__restrict__ nodes, const double2 *__restrict__ low,
                                                     uint32_t S, const uint32_t *__restrict__ grid_count,
                                                     uint32_t gc, uint32_t delay, double two_r, ExactCtx ex,
                                                     uint8_t *__restrict__ flags, uint32_t *__restrict__ aux,
                                                     uint32_t *__restrict__ newgid, uint32_t *__restrict__ cand,
                                                     DevCounters *cnt) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const DNode n = nodes[s];
        uint8_t f = kEvNone;
        if (n.type == kLeaf) {
            const uint32_t c = grid_count[n.gid];
            bool cond = false;
            if (c > gc) {
                const double2 lo = low[s];
                cond = width_gt_exact(lo.x, kdbl(n.khx), lo.y, two_r, ex);
            }
            int16_t of = 0;
            if (cond) {
                of = (int16_t)(n.of + 1);
                if ((uint32_t)of >= delay) {
                    f = kEvSplit;
                    of = 0;
                }
            }
            if (of != n.of) nodes[s].of = of;
        } else if (n.type == kBranch) {
            bool ok = true, has_branch = false;
            uint32_t sum = 0;
            for (int i = 0; i < 4; ++i) {
                const uint32_t ch = n.child[i];
                const DNode cn = nodes[ch];
                if (cn.type == kLeaf) sum += grid_count[cn.gid];
                else if (cn.type == kBranch && ch < s) has_branch = true;
                else ok = false;
            }
            int16_t uf = 0;
            if (ok && !has_branch) {
                if (sum < gc) {
                    uf = (int16_t)(n.uf + 1);
                    if ((uint32_t)uf >= delay) {
                        f = kEvMerge;
                        uf = 0;
                        newgid[s] = nodes[n.child[3]].gid;
                    }
                }
                if (uf != n.uf) nodes[s].uf = uf;
            } else if (ok) {
                f = kEvCand;
                aux[s] = sum;
                uint32_t idx = atomicAdd(&cnt->n_cand, 1u);
                cand[idx] = s;
            } else if (n.uf != 0) {
                nodes[s].uf = 0;
            }
        }
        flags[s] = f;
    }
}

/* bottom-up resolution of merge candidates (branches with branch children of
 * smaller slot); at most tree-depth rounds */
__global__ void __launch_bounds__(1024) k_sch_cascade(DNode *__restrict__ nodes, uint8_t *__restrict__ flags,
                                                      const uint32_t *__restrict__ aux, uint32_t *__restrict__ newgid,
                                                      const uint32_t *__restrict__ cand, uint32_t gc, uint32_t delay,
                                                      DevCounters *cnt) {
    __shared__ int changed;
    const uint32_t nc = cnt->n_cand;
    for (int round = 0; round < 80; ++round) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) {
            const uint32_t g = cand[i];
            if ((flags[g] & 3) != kEvCand) continue;
            const DNode n = nodes[g];
            bool all_merge = true, resolved = true;
            for (int k = 0; k < 4; ++k) {
                const uint32_t ch = n.child[k];
                const uint8_t cf = flags[ch] & 3;
                if (nodes[ch].type != kBranch) continue;   /* a leaf child */
                if (cf == kEvMerge) continue;
                if (cf == kEvCand) resolved = false;
                else all_merge = false;
            }
            if (!all_merge) {
                flags[g] = kEvNone;
                if (n.uf != 0) nodes[g].uf = 0;
                changed = 1;
            } else if (resolved) {
                int16_t uf = 0;
                uint8_t f = kEvNone;
                if (aux[g] < gc) {
                    uf = (int16_t)(n.uf + 1);
                    if ((uint32_t)uf >= delay) {
                        f = kEvMerge;
                        uf = 0;
                        const uint32_t c3 = n.child[3];
                        newgid[g] = (flags[c3] & 3) == kEvMerge ? newgid[c3] : nodes[c3].gid;
                    }
                }
                if (uf != n.uf) nodes[g].uf = uf;
                __threadfence_block();
                flags[g] = f;
                changed = 1;
            }
        }
        __syncthreads();
        if (!changed) break;
    }
    /* anything still unresolved cannot merge */
    for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) {
        const uint32_t g = cand[i];
        if ((flags[g] & 3) == kEvCand) flags[g] = kEvNone;
    }
}

/* mark the children of merged branches as freed (a merged child must not
 * become a leaf again) and count events */
__global__ void __launch_bounds__(256) k_sch_mark(const DNode *__restrict__ nodes, uint8_t *__restrict__ flags,
                                                  uint32_t S, uint32_t *__restrict__ is_event, DevCounters *cnt) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const uint8_t f = flags[s] & 3;
        uint32_t ev = 0;
        if (f == kEvMerge) {
            for (int k = 0; k < 4; ++k) {
                const uint32_t ch = nodes[s].child[k];
                if ((flags[ch] & 3) == kEvMerge) atomicOr(reinterpret_cast<unsigned int *>(flags + (ch & ~3u)),
                                                          (unsigned int)kEvFreed << (8 * (ch & 3u)));
            }
            ev = 1;
            atomicAdd(&cnt->merges, 1u);
        } else if (f == kEvSplit) {
            ev = 1;
            atomicAdd(&cnt->splits, 1u);
        }
        is_event[s] = ev;
    }
}

__global__ void __launch_bounds__(256) k_sch_compact(const uint32_t *__restrict__ is_event,
                                                     const uint32_t *__restrict__ pos, uint32_t S,
                                                     uint32_t *__restrict__ events, DevCounters *cnt) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x)
        if (is_event[s]) events[pos[s]] = s;
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt->n_events = pos[S];
}

/* per-event data for the stack replay: for a merge, its four children and
 * the grid ids they hold at that point of the pass; for a split, the parent's
 * grid id */
__global__ void __launch_bounds__(256) k_sch_evdata(const DNode *__restrict__ nodes, const uint8_t *__restrict__ flags,
                                                    const uint32_t *__restrict__ newgid,
                                                    const uint32_t *__restrict__ events, uint4 *__restrict__ evdata,
                                                    const DevCounters *cnt) {
    const uint32_t E = cnt->n_events;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t s = events[i];
        const DNode n = nodes[s];
        if ((flags[s] & 3) == kEvMerge) {
            uint32_t cg[4];
            for (int k = 0; k < 4; ++k) {
                const uint32_t ch = n.child[k];
                cg[k] = (flags[ch] & 3) == kEvMerge ? newgid[ch] : nodes[ch].gid;
            }
            evdata[2 * i] = make_uint4(n.child[0], n.child[1], n.child[2], n.child[3]);
            evdata[2 * i + 1] = make_uint4(cg[0], cg[1], cg[2], cg[3]);
        } else {
            evdata[2 * i] = make_uint4(0xffffffffu, 0, 0, 0); /* split marker */
            evdata[2 * i + 1] = make_uint4(n.gid, 0, 0, 0);
        }
    }
}

constexpr int kStackThreads = 1024;
constexpr uint32_t kChunk = 512;

/* replay of schema_stack / grids_stack operations in event order.  Output per
 * split event: child slots and child grid ids (into evdata, overwritten) */
__global__ void __launch_bounds__(kStackThreads) k_sch_stacks(uint32_t *__restrict__ sstack, uint32_t *__restrict__ gstack,
                                                              uint32_t S, uint32_t G, uint4 *__restrict__ evdata,
                                                              int32_t *__restrict__ levels, uint32_t win_cap,
                                                              DevCounters *cnt) {
    extern __shared__ uint32_t sm[];
    __shared__ uint4 chunk[2 * kChunk];
    __shared__ int32_t lv[kChunk];
    __shared__ int32_t s_min, s_max, s_carry;
    __shared__ uint32_t s_ws[32];
    const uint32_t E = cnt->n_events;
    if (E == 0) return;
    /* 1. level before each event (+1 split, -1 merge) and the range */
    if (threadIdx.x == 0) { s_min = 0; s_max = 0; s_carry = 0; }
    __syncthreads();
    for (uint32_t base = 0; base < E; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        int32_t d = 0;
        if (i < E) d = (evdata[2 * i].x == 0xffffffffu) ? 1 : -1;
        /* inclusive scan of d (signed) */
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        int32_t x = d;
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_ws[wid] = (uint32_t)x;
        __syncthreads();
        if (wid == 0) {
            int32_t v = lane < (int)(blockDim.x >> 5) ? (int32_t)s_ws[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int32_t y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += y;
            }
            s_ws[lane] = (uint32_t)v;
        }
        __syncthreads();
        const int32_t incl = s_carry + (wid ? (int32_t)s_ws[wid - 1] : 0) + x;
        const int32_t before = incl - d;
        if (i < E) {
            levels[i] = before;
            atomicMin(&s_min, before);
            atomicMax(&s_max, before);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_carry += (int32_t)s_ws[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    const int64_t ssi0 = cnt->ssi, gsi0 = cnt->gsi;
    const int64_t s_lo = ssi0 + 4 * (int64_t)s_min - 4, s_hi = ssi0 + 4 * (int64_t)s_max + 4;
    const int64_t g_lo = gsi0 + 3 * (int64_t)s_min - 4, g_hi = gsi0 + 3 * (int64_t)s_max + 3;
    if (s_lo < 0 || s_hi > (int64_t)S || g_lo < 0 || g_hi > (int64_t)G) {
        if (threadIdx.x == 0) {
            atomicOr(&cnt->error_flags, GLINT_EF_SCHEMA_STACK);
            cnt->n_events = 0; /* nothing is applied */
        }
        return;
    }
    const uint32_t s_n = (uint32_t)(s_hi - s_lo), g_n = (uint32_t)(g_hi - g_lo);
    const bool in_smem = (s_n + g_n) <= win_cap;
    uint32_t *ws = in_smem ? sm : sstack + s_lo;
    uint32_t *wg = in_smem ? sm + s_n : gstack + g_lo;
    if (in_smem) {
        for (uint32_t i = threadIdx.x; i < s_n; i += blockDim.x) ws[i] = sstack[s_lo + i];
        for (uint32_t i = threadIdx.x; i < g_n; i += blockDim.x) wg[i] = gstack[g_lo + i];
    } else if (threadIdx.x == 0) {
        atomicOr(&cnt->error_flags, GLINT_EF_SCHEMA_WINDOW);
    }
    __syncthreads();
    /* 2. replay in chunks */
    for (uint32_t cb = 0; cb < E; cb += kChunk) {
        const uint32_t ce = min(E, cb + kChunk);
        for (uint32_t i = cb + threadIdx.x; i < ce; i += blockDim.x) {
            chunk[2 * (i - cb)] = evdata[2 * i];
            chunk[2 * (i - cb) + 1] = evdata[2 * i + 1];
            lv[i - cb] = levels[i];
        }
        __syncthreads();
        /* the serial part touches shared memory only */
        if (threadIdx.x == 0) {
            for (uint32_t i = cb; i < ce; ++i) {
                const int32_t k = lv[i - cb];
                const int64_t sp = ssi0 + 4 * (int64_t)k - s_lo;  /* schema_stack_index in the window */
                const int64_t gp = gsi0 + 3 * (int64_t)k - g_lo;  /* grids_stack_index in the window */
                uint4 &a = chunk[2 * (i - cb)];
                uint4 &b = chunk[2 * (i - cb) + 1];
                if (a.x == 0xffffffffu) {
                    /* split_node (filter.cpp:343-358) */
                    const uint32_t pg = b.x;
                    wg[gp - 1] = pg;
                    a = make_uint4(ws[sp], ws[sp + 1], ws[sp + 2], ws[sp + 3]);
                    b = make_uint4(pg, wg[gp], wg[gp + 1], wg[gp + 2]);
                } else {
                    /* merge_node (filter.cpp:323-334) */
                    ws[sp - 1] = a.x;
                    ws[sp - 2] = a.y;
                    ws[sp - 3] = a.z;
                    ws[sp - 4] = a.w;
                    wg[gp - 1] = b.x;
                    wg[gp - 2] = b.y;
                    wg[gp - 3] = b.z;
                    wg[gp - 4] = b.w;
                }
            }
        }
        __syncthreads();
        for (uint32_t i = cb + threadIdx.x; i < ce; i += blockDim.x) {
            evdata[2 * i] = chunk[2 * (i - cb)];
            evdata[2 * i + 1] = chunk[2 * (i - cb) + 1];
        }
        __syncthreads();
    }
    if (in_smem) {
        for (uint32_t i = threadIdx.x; i < s_n; i += blockDim.x) sstack[s_lo + i] = ws[i];
        for (uint32_t i = threadIdx.x; i < g_n; i += blockDim.x) gstack[g_lo + i] = wg[i];
    }
    if (threadIdx.x == 0) {
        cnt->ssi = (unsigned)(ssi0 + 4 * (int64_t)s_carry);
        cnt->gsi = (unsigned)(gsi0 + 3 * (int64_t)s_carry);
    }
}

__global__ void __launch_bounds__(256) k_sch_apply_merge(DNode *__restrict__ nodes, const uint8_t *__restrict__ flags,
                                                         const uint32_t *__restrict__ newgid,
                                                         const uint32_t *__restrict__ events, const uint4 *evdata,
                                                         uint32_t *__restrict__ grid_count, const DevCounters *cnt) {
    const uint32_t E = cnt->n_events;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint4 a = evdata[2 * i];
        if (a.x == 0xffffffffu || (flags[events[i]] & 3) != kEvMerge) continue;
        const uint32_t g = events[i];
        /* merge_node zeroes the counters of the grids it frees (filter.cpp:331) */
        const uint4 cg = evdata[2 * i + 1];
        grid_count[cg.x] = 0;
        grid_count[cg.y] = 0;
        grid_count[cg.z] = 0;
        grid_count[cg.w] = 0;
        nodes[a.x].type = kInvalid;
        nodes[a.y].type = kInvalid;
        nodes[a.z].type = kInvalid;
        nodes[a.w].type = kInvalid;
        if (!(flags[g] & kEvFreed)) {
            nodes[g].type = kLeaf;
            nodes[g].gid = newgid[g];
        }
    }
}

__global__ void __launch_bounds__(256) k_sch_apply_split(DNode *__restrict__ nodes, double2 *__restrict__ low,
                                                         IBox *__restrict__ ibox, Frame fr,
                                                         const uint8_t *__restrict__ flags,
                                                         const uint32_t *__restrict__ events, const uint4 *evdata,
                                                         uint32_t *__restrict__ grid_count, const DevCounters *cnt) {
    const uint32_t E = cnt->n_events;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t p = events[i];
        if ((flags[p] & 3) != kEvSplit) continue;
        const uint4 cs = evdata[2 * i], gs = evdata[2 * i + 1];
        /* split_node zeroes the counters of the children's grids (filter.cpp:359) */
        grid_count[gs.x] = 0;
        grid_count[gs.y] = 0;
        grid_count[gs.z] = 0;
        grid_count[gs.w] = 0;
        const DNode pn = nodes[p];
        const double2 pl = low[p];
        const double pmx = kdbl(pn.kmx), pmy = kdbl(pn.kmy);
        /* split_node (tracing/filter.cpp:347-370): children are the parent's
         * quadrants, offset by half the parent's extent; the boxes are also
         * kept in fixed point for the filter's screening */
        const double xhalf = __dsub_rn(pmx, pl.x);
        const double yhalf = __dsub_rn(pmy, pl.y);
        const uint32_t ch[4] = {cs.x, cs.y, cs.z, cs.w};
        const uint32_t gg[4] = {gs.x, gs.y, gs.z, gs.w};
        for (int k = 0; k < 4; ++k) {
            const double ox = (k % 2 == 1) ? xhalf : 0.0;
            const double oy = (k / 2 == 1) ? yhalf : 0.0;
            DNode c;
            const double lx = __dadd_rn(pl.x, ox);
            const double ly = __dadd_rn(pl.y, oy);
            const double hx = __dadd_rn(pmx, ox);
            const double hy = __dadd_rn(pmy, oy);
            c.khx = dkey(hx);
            c.khy = dkey(hy);
            c.kmx = dkey(__dmul_rn(__dadd_rn(lx, hx), 0.5));
            c.kmy = dkey(__dmul_rn(__dadd_rn(ly, hy), 0.5));
            ibox[ch[k]] = fx_box(lx, ly, hx, hy, fr);
            c.child[0] = c.child[1] = c.child[2] = c.child[3] = 0;
            c.gid = gg[k];
            c.type = kLeaf;
            c.pad0 = 0;
            c.level = (int16_t)(pn.level + 1);
            c.of = 0;
            c.uf = 0;
            c.pad1 = 0;
            nodes[ch[k]] = c;
            low[ch[k]] = make_double2(lx, ly);
        }
        DNode q = pn;
        q.type = kBranch;
        q.child[0] = ch[0];
        q.child[1] = ch[1];
        q.child[2] = ch[2];
        q.child[3] = ch[3];
        nodes[p] = q;
    }
}

size_t schema_stack_smem(uint32_t win_cap) { return (size_t)win_cap * sizeof(uint32_t); }
constexpr uint32_t kWinCap = 40000; /* window entries in shared memory (160 KB) */

cudaError_t launch_schema_update(glint_ctx *c, cudaStream_t s, void *scan_tmp) {
    const uint32_t S = c->S;
    ExactCtx ex = make_exact(c);
    cudaMemsetAsync(&c->d_cnt->n_cand, 0, sizeof(unsigned int), s);
    k_sch_collect<<<grid_for(S, 256, 152u * 8u), 256, 0, s>>>(c->d_nodes, c->d_low, S, c->d_grid_count,
                                                               c->cfg.grid_capacity, c->cfg.schema_update_delay,
                                                               2.0 * c->cfg.reach_distance, ex, c->d_split,
                                                               c->d_evscan, c->d_newgid, c->d_cand, c->d_cnt);
    k_sch_cascade<<<1, 1024, 0, s>>>(c->d_nodes, c->d_split, c->d_evscan, c->d_newgid, c->d_cand,
                                     c->cfg.grid_capacity, c->cfg.schema_update_delay, c->d_cnt);
    k_sch_mark<<<grid_for(S, 256, 152u * 8u), 256, 0, s>>>(c->d_nodes, c->d_split, S, c->d_events, c->d_cnt);
    scan_u32(c->d_events, c->d_evpos, S, scan_tmp, s);
    k_sch_compact<<<grid_for(S, 256, 152u * 8u), 256, 0, s>>>(c->d_events, c->d_evpos, S, c->d_evlist, c->d_cnt);
    k_sch_evdata<<<152, 256, 0, s>>>(c->d_nodes, c->d_split, c->d_newgid, c->d_evlist, c->d_evdata, c->d_cnt);
    k_sch_stacks<<<1, kStackThreads, schema_stack_smem(kWinCap), s>>>(c->d_sstack, c->d_gstack, S, c->G, c->d_evdata,
                                                                       c->d_evlevel, kWinCap, c->d_cnt);
    k_sch_apply_merge<<<152, 256, 0, s>>>(c->d_nodes, c->d_split, c->d_newgid, c->d_evlist, c->d_evdata,
                                          c->d_grid_count, c->d_cnt);
    k_sch_apply_split<<<152, 256, 0, s>>>(c->d_nodes, c->d_low, c->d_ibox, c->frame, c->d_split, c->d_evlist,
                                          c->d_evdata,
                                          c->d_grid_count, c->d_cnt);
    return cudaGetLastError();
}

void schema_set_attributes() {
    cudaFuncSetAttribute(k_sch_stacks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)schema_stack_smem(kWinCap));
}

} // namespace glint
