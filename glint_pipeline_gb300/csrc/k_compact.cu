/*
 * k_compact.cu -- compaction of kept blocks on the device: merge_dump
 * (tools/compaction.cpp:729-1215), which merges consecutive contact-tracing
 * blocks into one block of split_num^2 CTFs.
 *
 * The reference walks every object of every source block on the host.  Here
 * each stage is one pass over flat arrays:
 *   parse     one thread per source CTF key: CTF::parse_key and
 *             new_parse_mbr_f_box (tracing/step_merge.cpp:347-398), the end
 *             made absolute; a key whose object its block marks oversize is
 *             flagged for the extra oversize list (:797-806)
 *   order     stable radix sort of (extra, oid, target): each object's keys
 *             become one run ordered by target, equal targets in source
 *             order (cmp_ki, :92-97, 819-824)
 *   objects   one thread per object over its run: box (f_box::update), start
 *             limits, the middle of its box (:826-838)
 *   STR       stable radix sorts by x middle, then by y middle inside each x
 *             part (compare_two_level / compare_y, :839-889), and the sid of
 *             every position below split_index (:900-917)
 *   CTFs      objects ordered by (CTF, oid); each CTF's list is filled to its
 *             size with object 0, whose keys then lead the CTF (:908-938);
 *             box and start limits per CTF, get_ctf_bits on the host
 *             (:960-1004)
 *   pack      one thread per output key: its bitmap cells (:1010-1040) and
 *             its packed key with end + end_time_min (:1045-1063)
 *   oversize  the source buffers and the extra list concatenated and sorted
 *             stably by the 128-bit key, which is the reference's
 *             smallest-head merge for buffers in key order (:1079-1127)
 * Where merge_dump leaves ties to std::sort, the order here is the stable one
 * named above.
 */
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "glint_internal.cuh"
#include "store_codec.cuh"

namespace glint {
namespace {

constexpr int kOidBit = 26;                  /* OID_BIT, util/util.h:49 */
constexpr uint64_t kBitBytes = 256 * 256 / 8; /* one CTF's bitmap slot */
constexpr unsigned long long kExtraFlag = 1ull << 52;
constexpr uint64_t kCellLoopMax = 1ull << 20;

typedef unsigned __int128 u128;

struct SrcBlock {
    const uint8_t *keys;
    const glint_ctf_meta *ctfs;
    const unsigned long long *key_index, *byte_index;
    const uint16_t *sids;
    const uint3 *toff;          /* [C] offsets of each CTF's decode tables */
    unsigned long long base;    /* first record of the block */
    unsigned long long key_bytes;
    uint32_t C, pad;
};

/* one parsed CTF key */
struct Rec {
    uint32_t oid, target, duration, end;   /* end absolute */
    float4 box;
};

enum : uint32_t {
    kErrOid = 0,      /* a key's object id beyond num_objects */
    kErrOrder = 1,    /* a source oversize buffer out of key order */
    kErrCells = 2,    /* a key box over too many bitmap cells */
    kExtraCount = 3,  /* keys for the extra oversize list */
    kNoSid = 4,       /* source oversize keys without sid bits */
    kExtraOrder = 5,  /* the extra list out of full-key order */
    kNumCounters = 6
};

__device__ inline uint32_t last_le(const unsigned long long *a, uint32_t n, unsigned long long v) {
    /* the last i with a[i] <= v (a ascending, a[0] <= v) */
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

/* decode tables of one CTF (new_parse_mbr_f_box, tracing/step_merge.cpp:381-398):
 * the low corner's coordinates for every quantised value, rounded to float,
 * and the edge offsets in double; the box is then b0 = T0[l0], b2 =
 * float(double(b0) + E[x]), the reference's operations in its order */
__global__ void k_cmp_tables(const glint_ctf_meta *__restrict__ ctfs, const uint3 *__restrict__ toff,
                             float *__restrict__ tf, double *__restrict__ td) {
    const uint32_t j = blockIdx.x;
    const glint_ctf_meta m = ctfs[j];
    const uint3 o = toff[j];
    const uint64_t me = (1ull << m.edge_bit) - 1, my = (1ull << m.low_y_bit) - 1, mx = (1ull << m.low_x_bit) - 1;
    const float ex = __fsub_rn(m.ctf_mbr[2], m.ctf_mbr[0]), ey = __fsub_rn(m.ctf_mbr[3], m.ctf_mbr[1]);
    const float le = ex < ey ? ey : ex;
    for (uint64_t v = threadIdx.x; v <= mx; v += blockDim.x)
        tf[o.x + v] = __double2float_rn(
            __dadd_rn((double)m.ctf_mbr[0], __dmul_rn(__ddiv_rn(__ull2double_rn(v), __ull2double_rn(mx)), (double)ex)));
    for (uint64_t v = threadIdx.x; v <= my; v += blockDim.x)
        tf[o.y + v] = __double2float_rn(
            __dadd_rn((double)m.ctf_mbr[1], __dmul_rn(__ddiv_rn(__ull2double_rn(v), __ull2double_rn(my)), (double)ey)));
    for (uint64_t v = threadIdx.x; v <= me; v += blockDim.x)
        td[o.z + v] = __dmul_rn(__ddiv_rn(__ull2double_rn(v), __ull2double_rn(me)), (double)le);
}


__global__ void __launch_bounds__(256) k_cmp_parse(const SrcBlock *__restrict__ src, uint32_t nsrc, uint64_t R,
                                                   uint32_t N, const float *__restrict__ tf,
                                                   const double *__restrict__ td, Rec *__restrict__ recs,
                                                   unsigned long long *__restrict__ skey, uint32_t *__restrict__ sval,
                                                   unsigned long long *__restrict__ counters) {
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < R; g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t i = 0;
        while (i + 1 < nsrc && src[i + 1].base <= g) ++i;
        const SrcBlock b = src[i];
        const unsigned long long k = g - b.base;
        const uint32_t j = last_le(b.key_index, b.C, k);
        const glint_ctf_meta m = b.ctfs[j];
        const uint32_t kb = m.key_bit / 8;
        u128 v = load_key(b.keys + b.byte_index[j] + (k - b.key_index[j]) * kb, kb, b.keys + b.key_bytes);
        /* CTF::parse_key */
        uint64_t vm = (uint64_t)(v & (((u128)1 << m.mbr_bit) - 1));
        v >>= m.mbr_bit;
        Rec r;
        r.end = (uint32_t)(v & ((1ull << m.end_bit) - 1));
        v >>= m.end_bit;
        r.duration = (uint32_t)(v & ((1ull << m.duration_bit) - 1));
        v >>= m.duration_bit;
        r.target = (uint32_t)(v & ((1ull << m.id_bit) - 1));
        v >>= m.id_bit;
        /* the flush writes its whole (sid, oid) field above the target, and
         * the packed bytes keep sid bits when key_bit rounds up past the id
         * (N > 2^19): the id is read with id_bit bits, as
         * CTF::ctf_get_key_oid (tracing/step_merge.cpp:331-333) reads it */
        r.oid = (uint32_t)(v & ((1ull << m.id_bit) - 1));
        r.end += m.end_time_min;
        /* the box from the CTF's decode tables */
        const uint3 o = b.toff[j];
        const uint64_t me = (1ull << m.edge_bit) - 1, my = (1ull << m.low_y_bit) - 1, mx = (1ull << m.low_x_bit) - 1;
        const uint64_t y = vm & me;
        vm >>= m.edge_bit;
        const uint64_t x = vm & me;
        vm >>= m.edge_bit;
        const uint64_t l1 = vm & my;
        vm >>= m.low_y_bit;
        const uint64_t l0 = vm & mx;
        const float b0 = tf[o.x + l0], b1 = tf[o.y + l1];
        const float b2 = __double2float_rn(__dadd_rn((double)b0, td[o.z + x]));
        const float b3 = __double2float_rn(__dadd_rn((double)b1, td[o.z + y]));
        r.box = make_float4(b0, b1, b2, b3);
        recs[g] = r;
        sval[g] = (uint32_t)g;
        if (r.oid >= N || r.target >= (1u << kOidBit)) {
            atomicAdd(&counters[kErrOid], 1ull);
            skey[g] = kExtraFlag | ((unsigned long long)((1u << kOidBit) - 1) << kOidBit);
            continue;
        }
        const bool extra = b.sids[r.oid] == 1;
        if (extra) atomicAdd(&counters[kExtraCount], 1ull);
        skey[g] = (extra ? kExtraFlag : 0ull) | ((unsigned long long)r.oid << kOidBit) | r.target;
    }
}

/* the records in sorted order */
__global__ void k_cmp_permute(uint64_t n, const uint32_t *__restrict__ sidx, const Rec *__restrict__ recs,
                              Rec *__restrict__ out) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x)
        out[p] = recs[sidx[p]];
}

/* each object's run [first, end) in the sorted order */
__global__ void k_cmp_runs(const unsigned long long *__restrict__ skey, uint64_t n, uint32_t *__restrict__ rfirst,
                           uint32_t *__restrict__ rend) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long o = skey[p] >> kOidBit;
        if (p == 0 || (skey[p - 1] >> kOidBit) != o) rfirst[o] = (uint32_t)p;
        if (p + 1 == n || (skey[p + 1] >> kOidBit) != o) rend[o] = (uint32_t)(p + 1);
    }
}

/* ave_loc holds a float widened to double, so the float's order is the
 * double's; -0 and +0 compare equal */
__device__ inline unsigned long long order_key(float v) {
    if (v == 0.0f) v = 0.0f;
    const uint32_t u = __float_as_uint(v);
    return (u >> 31) ? (~u & 0xffffffffu) : (u | 0x80000000u);
}

/* per object: key count, box (f_box::update), start limits, class (0 none, 1
 * oversize in a source block, 2 CTF keys) and the middles of its box */
__global__ void k_cmp_objects(uint32_t N, const uint32_t *__restrict__ rfirst, const uint32_t *__restrict__ rend,
                              const Rec *__restrict__ prec,
                              const SrcBlock *__restrict__ src, uint32_t nsrc, uint32_t *__restrict__ nkeys,
                              float4 *__restrict__ obox, uint2 *__restrict__ ostart, uint8_t *__restrict__ cls,
                              uint32_t *__restrict__ is2, unsigned long long *__restrict__ xkey,
                              unsigned long long *__restrict__ ykey) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x) {
        const uint32_t f = rfirst[o], e = rend[o];
        const uint32_t n = e > f ? e - f : 0u;
        float4 a = make_float4(100000.0f, 100000.0f, -100000.0f, -100000.0f);
        uint32_t smin = 1u << 30, smax = 1u;
        for (uint32_t p = f; p < e; ++p) {
            const Rec r = prec[p];
            if (a.x > r.box.x) a.x = r.box.x;
            if (a.z < r.box.z) a.z = r.box.z;
            if (a.y > r.box.y) a.y = r.box.y;
            if (a.w < r.box.w) a.w = r.box.w;
            const uint32_t st = r.end - r.duration;
            smin = st < smin ? st : smin;
            smax = smax < st ? st : smax;
        }
        uint8_t c = n ? 2 : 0;
        if (!n)
            for (uint32_t i = 0; i < nsrc; ++i)
                if (src[i].sids[o] == 1) c = 1;
        nkeys[o] = n;
        obox[o] = a;
        ostart[o] = make_uint2(smin, smax);
        cls[o] = c;
        is2[o] = c == 2;
        /* ave_loc: float halves added in float (then widened to double) */
        xkey[o] = order_key(__fadd_rn(__fdiv_rn(a.x, 2.0f), __fdiv_rn(a.z, 2.0f)));
        ykey[o] = order_key(__fadd_rn(__fdiv_rn(a.y, 2.0f), __fdiv_rn(a.w, 2.0f)));
    }
}

/* the objects marked 2 in id order, with their x keys */
__global__ void k_cmp_list2(uint32_t N, const uint32_t *__restrict__ is2, const uint32_t *__restrict__ pos,
                            const unsigned long long *__restrict__ xkey, unsigned long long *__restrict__ lk,
                            uint32_t *__restrict__ lv) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x)
        if (is2[o]) {
            lk[pos[o]] = xkey[o];
            lv[pos[o]] = o;
        }
}

/* y keys of the x-sorted positions; the key sort by part follows */
__global__ void k_cmp_ykeys(uint32_t S, const uint32_t *__restrict__ xorder, const unsigned long long *__restrict__ ykey,
                            unsigned long long *__restrict__ yk, uint32_t *__restrict__ yv) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < S; p += gridDim.x * blockDim.x) {
        yk[p] = ykey[xorder[p]];
        yv[p] = p;
    }
}

/* part of every position: p / x_part for p < split_index (the last part
 * runs to split_index), split_num for split_index itself, which stays last */
__global__ void k_cmp_parts(uint32_t S, uint32_t split, uint32_t x_part, uint32_t s, const uint32_t *__restrict__ yv,
                            unsigned long long *__restrict__ pk) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
        const uint32_t p = yv[i];
        uint32_t part = p < split ? p / x_part : s;
        if (p < split && part > s - 1) part = s - 1;
        pk[i] = part;
    }
}

/* positions [0, split_index) get their CTF (merge_dump :900-917) */
__global__ void k_cmp_assign(uint32_t split, uint32_t x_part, uint32_t y_part, uint32_t s,
                             const uint32_t *__restrict__ yv, const uint32_t *__restrict__ xorder,
                             uint16_t *__restrict__ sids, uint32_t *__restrict__ ctf_of) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < split; i += gridDim.x * blockDim.x) {
        const uint32_t o = xorder[yv[i]];
        const uint32_t xi = i / x_part, yi = (i % x_part) / y_part;
        const uint32_t c = xi * s + yi;
        sids[o] = (uint16_t)(c + 2);
        ctf_of[o] = c;
    }
}

__global__ void k_cmp_placed(uint32_t N, const uint32_t *__restrict__ ctf_of, uint32_t *__restrict__ flag) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x)
        flag[o] = ctf_of[o] != 0xffffffffu;
}

/* the placed objects in id order, keyed by CTF (a stable sort by CTF then
 * gives the (CTF, oid) order of the CTFs' object lists) */
__global__ void k_cmp_plist(uint32_t N, const uint32_t *__restrict__ ctf_of, const uint32_t *__restrict__ pos,
                            unsigned long long *__restrict__ ck, uint32_t *__restrict__ cv) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x) {
        const uint32_t c = ctf_of[o];
        if (c == 0xffffffffu) continue;
        ck[pos[o]] = c;
        cv[pos[o]] = o;
    }
}

__global__ void k_cmp_listn(uint32_t n, const uint32_t *__restrict__ olist, const uint32_t *__restrict__ nkeys,
                            uint32_t *__restrict__ nl, uint32_t *__restrict__ posof) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        nl[j] = nkeys[olist[j]];
        posof[olist[j]] = j;
    }
}

/* box and start limits of CTF c over its objects (and object 0 when its
 * list is padded); the reference folds keys with std::min / std::max */
__global__ void __launch_bounds__(256) k_cmp_limits(const unsigned long long *__restrict__ cstart,
                                                    const uint32_t *__restrict__ olist, const float4 *__restrict__ obox,
                                                    const uint2 *__restrict__ ostart,
                                                    const unsigned long long *__restrict__ pad, uint32_t n0,
                                                    float4 *__restrict__ lim, uint2 *__restrict__ slim) {
    __shared__ float4 sb[256];
    __shared__ uint2 ss[256];
    const uint32_t c = blockIdx.x;
    float4 a = make_float4(100000.0f, 100000.0f, -100000.0f, -100000.0f);
    uint32_t smin = 1u << 30, smax = 1u;
    auto take = [&](const float4 &b, const uint2 &st) {
        if (b.x < a.x) a.x = b.x;
        if (b.y < a.y) a.y = b.y;
        if (a.z < b.z) a.z = b.z;
        if (a.w < b.w) a.w = b.w;
        smin = st.x < smin ? st.x : smin;
        smax = smax < st.y ? st.y : smax;
    };
    if (threadIdx.x == 0 && pad[c] && n0) take(obox[0], ostart[0]);
    for (unsigned long long j = cstart[c] + threadIdx.x; j < cstart[c + 1]; j += blockDim.x) {
        const uint32_t o = olist[j];
        take(obox[o], ostart[o]);
    }
    sb[threadIdx.x] = a;
    ss[threadIdx.x] = make_uint2(smin, smax);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t t = 1; t < blockDim.x; ++t) take(sb[t], ss[t]);
        lim[c] = a;
        slim[c] = make_uint2(smin, smax);
    }
}

struct PackArgs {
    const glint_ctf_meta *ctfs;
    const unsigned long long *key_index, *byte_index; /* [C + 1] */
    const unsigned long long *cstart;                  /* [C + 1] object-list start of each CTF */
    const unsigned long long *pad;                     /* [C] object-list entries filled with object 0 */
    const unsigned long long *padk;                    /* [C + 1] prefix of pad * n0: the repeated keys */
    const uint32_t *escan;                             /* [placed + 1] keys before each listed object */
    const uint32_t *posof, *rfirst, *ctf_of;
    const unsigned long long *obase;                   /* [N] a placed object's first key in the block */
    const Rec *prec;                                   /* records in (oid, target) order */
    uint8_t *out;
    uint32_t *bits;
    unsigned long long *counters;
    uint64_t n;                                        /* records (or repeated keys) to emit */
    uint32_t C, n0;
};

/* every placed object's records into output order (a placed object's keys
 * follow object 0's repeats and the keys of the CTF's objects before it),
 * whole 32-byte records so the scattered writes fill their sectors */
__global__ void __launch_bounds__(256) k_cmp_place(PackArgs a, Rec *__restrict__ out) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < a.n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const Rec r = a.prec[p];
        if (a.ctf_of[r.oid] == 0xffffffffu) continue; /* the object STR leaves unplaced */
        out[a.obase[r.oid] + (p - a.rfirst[r.oid])] = r;
    }
}

/* object 0's repeats at the front of the CTFs whose object lists STR leaves
 * short */
__global__ void __launch_bounds__(256) k_cmp_place_pad(PackArgs a, Rec *__restrict__ out) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < a.n;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = last_le(a.padk, a.C, t);
        const unsigned long long q = t - a.padk[c];
        out[a.key_index[c] + q] = a.prec[a.rfirst[0] + q % a.n0];
    }
}

/* one block per chunk of a CTF's keys, in output order: consecutive threads
 * write consecutive packed keys, and the chunk's bitmap cells (:1018-1038)
 * are set in shared memory and OR-ed into the CTF's bitmap once */
constexpr uint32_t kPackChunk = 16384;
__global__ void __launch_bounds__(256) k_cmp_pack(PackArgs a, const Rec *__restrict__ ordered,
                                                  const uint2 *__restrict__ chunks) {
    __shared__ uint32_t sbits[kBitBytes / 4];
    __shared__ uint8_t stage[8][32 * 16];  /* each warp's 32 packed keys */
    const uint2 ch = chunks[blockIdx.x];   /* (CTF, first key of the chunk within it) */
    const uint32_t c = ch.x;
    const glint_ctf_meta m = a.ctfs[c];
    const unsigned long long k0 = a.key_index[c], k1 = a.key_index[c + 1];
    const unsigned long long b = k0 + ch.y, e = b + kPackChunk < k1 ? b + kPackChunk : k1;
    const uint32_t words = ((uint32_t)m.x_grid * m.y_grid + 31) / 32;
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) sbits[i] = 0;
    __syncthreads();
    const float ex = __fsub_rn(m.ctf_mbr[2], m.ctf_mbr[0]), ey = __fsub_rn(m.ctf_mbr[3], m.ctf_mbr[1]);
    const float xg = (float)m.x_grid, yg = (float)m.y_grid;
    const uint32_t kb = m.key_bit / 8;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *st = stage[w];
    uint8_t *out = a.out + a.byte_index[c];
    for (unsigned long long t0 = b + (unsigned long long)w * 32; t0 < e; t0 += blockDim.x) {
        const unsigned long long t = t0 + lane;
        const bool valid = t < e;
        if (valid) {
            const Rec r = ordered[t];
            const uint32_t l0 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(r.box.x, m.ctf_mbr[0]), ex), xg));
            const uint32_t l1 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(r.box.y, m.ctf_mbr[1]), ey), yg));
            const uint32_t h0 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(r.box.z, m.ctf_mbr[0]), ex), xg));
            const uint32_t h1 = __float2uint_rz(__fmul_rn(__fdiv_rn(__fsub_rn(r.box.w, m.ctf_mbr[1]), ey), yg));
            uint64_t cells = 0;
            for (uint32_t mx = l0; mx <= h0 && mx < m.x_grid; ++mx)
                for (uint32_t ny = l1; ny <= h1 && ny < m.y_grid; ++ny) {
                    if (++cells > kCellLoopMax) {
                        atomicAdd(&a.counters[kErrCells], 1ull);
                        mx = h0;
                        break;
                    }
                    const uint32_t pb = mx + ny * m.x_grid, bit = 1u << (pb & 31);
                    /* an object's keys share cells: most are set already */
                    if (!(sbits[pb >> 5] & bit)) atomicOr(&sbits[pb >> 5], bit);
                }
            /* the key (:1049-1060), the end made absolute once more */
            const u128 vm = serialize_box(r.box, m);
            const u128 end = (u128)r.end + m.end_time_min;
            const u128 key = ((u128)r.oid << (m.id_bit + m.duration_bit + m.end_bit + m.mbr_bit)) +
                             ((u128)r.target << (m.duration_bit + m.end_bit + m.mbr_bit)) +
                             ((u128)r.duration << (m.end_bit + m.mbr_bit)) + (end << m.mbr_bit) + vm;
            put_key_bytes(st + lane * kb, key, kb);
        }
        __syncwarp();
        /* the warp's keys are one run of bytes: aligned words, edge bytes */
        const unsigned long long n = e - t0 < 32 ? e - t0 : 32;
        const uint32_t len = (uint32_t)n * kb;
        uint8_t *g = out + (t0 - k0) * kb;
        const uint32_t head = (uint32_t)((4 - ((uintptr_t)g & 3)) & 3) < len ? (uint32_t)((4 - ((uintptr_t)g & 3)) & 3)
                                                                                : len;
        const uint32_t nw = (len - head) / 4, tail0 = head + nw * 4;
        if ((uint32_t)lane < head) g[lane] = st[lane];
        for (uint32_t q = lane; q < nw; q += 32) {
            const uint8_t *sp = st + head + 4 * q;
            *(uint32_t *)(g + head + 4 * q) =
                (uint32_t)sp[0] | ((uint32_t)sp[1] << 8) | ((uint32_t)sp[2] << 16) | ((uint32_t)sp[3] << 24);
        }
        if ((uint32_t)lane < len - tail0) g[tail0 + lane] = st[tail0 + lane];
        __syncwarp();
    }
    __syncthreads();
    uint32_t *bits = a.bits + (uint64_t)c * (kBitBytes / 4);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x)
        if (sbits[i]) atomicOr(&bits[i], sbits[i]);
}

/* where each object's keys sit in the new block (its run of its own oid in
 * the CTF its sid names: object 0's repeats included, none for the object
 * STR leaves unplaced) */
__global__ void k_cmp_index(uint32_t N, const uint16_t *__restrict__ sids, const uint32_t *__restrict__ nkeys,
                            const uint32_t *__restrict__ posof, const unsigned long long *__restrict__ cstart,
                            const unsigned long long *__restrict__ key_index, const unsigned long long *__restrict__ pad,
                            const uint32_t *__restrict__ escan, const uint32_t *__restrict__ olist, uint32_t C,
                            uint32_t n0, uint32_t *__restrict__ first, uint32_t *__restrict__ count,
                            unsigned long long *__restrict__ obase) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x) {
        const uint32_t sid = sids[o];
        uint32_t f = 0, n = 0;
        if (sid >= 2 && sid - 2 < C) {
            const uint32_t c = sid - 2;
            const unsigned long long j = posof[o];
            const bool member = j >= cstart[c] && j < cstart[c + 1] && olist[j] == o;
            const unsigned long long padk = pad[c] * n0;
            if (member) {
                f = (uint32_t)(key_index[c] + padk + (escan[j] - escan[cstart[c]]));
                obase[o] = f;
                n = nkeys[o];
                if (o == 0) {
                    f = (uint32_t)key_index[c];
                    n += (uint32_t)padk;
                }
            } else if (o == 0 && padk) {
                f = (uint32_t)key_index[c];
                n = (uint32_t)padk;
            }
        }
        first[o] = f;
        count[o] = n;
    }
}

/* the oversize buffers one after another, then the extra list as
 * (oid, target, duration, end) keys without sid bits (:1090-1097) */
__global__ void k_cmp_ocat(const ulonglong2 *__restrict__ okeys, const float4 *__restrict__ oboxes, uint64_t n_src,
                           const Rec *__restrict__ prec, uint64_t extra_at,
                           uint64_t n_extra, unsigned long long *__restrict__ lo, unsigned long long *__restrict__ hi,
                           float4 *__restrict__ box, uint64_t at) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_src + n_extra;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < n_src) { /* n_src > 0 only with source keys */
            lo[at + i] = okeys[i].x;
            hi[at + i] = okeys[i].y;
            box[at + i] = oboxes[i];
        } else {
            const Rec r = prec[extra_at + (i - n_src)];
            lo[at + i] = ((unsigned long long)r.duration << 32) | r.end;
            hi[at + i] = ((unsigned long long)r.oid << kOidBit) | r.target;
            box[at + i] = r.box;
        }
    }
}

/* the smallest-head merge equals a stable sort for buffers in key order;
 * source keys without sid bits could interleave with the extra list */
__global__ void k_cmp_ocheck(const ulonglong2 *__restrict__ okeys, uint64_t n, unsigned long long *counters) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const ulonglong2 b = okeys[i];
        if ((b.y >> 52) == 0) atomicAdd(&counters[kNoSid], 1ull);
        if (i == 0) continue;
        const ulonglong2 a = okeys[i - 1];
        if (b.y < a.y || (b.y == a.y && b.x < a.x)) atomicAdd(&counters[kErrOrder], 1ull);
    }
}

/* the extra list (sorted by oid and target) in full-key order? */
__global__ void k_cmp_xcheck(const Rec *__restrict__ prec, uint64_t at, uint64_t n, unsigned long long *counters) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x + 1; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const Rec a = prec[at + i - 1], b = prec[at + i];
        if (a.oid == b.oid && a.target == b.target &&
            (b.duration < a.duration || (b.duration == a.duration && b.end < a.end)))
            atomicAdd(&counters[kExtraOrder], 1ull);
    }
}

__global__ void k_cmp_gather_hi(uint64_t n, const uint32_t *__restrict__ perm, const unsigned long long *__restrict__ hi,
                                unsigned long long *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = hi[perm[i]];
}

__global__ void k_cmp_ogather(uint64_t n, const uint32_t *__restrict__ perm, const unsigned long long *__restrict__ lo,
                              const unsigned long long *__restrict__ hi, const float4 *__restrict__ box,
                              ulonglong2 *__restrict__ okeys, float4 *__restrict__ oboxes) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = perm[i];
        okeys[i] = make_ulonglong2(lo[p], hi[p]);
        oboxes[i] = box[p];
    }
}

/* objects of sid 1: their first run in the merged buffer (the pid sits above
 * the target in the high word) */
__global__ void k_cmp_orun_first(const ulonglong2 *__restrict__ okeys, uint64_t n, uint32_t N,
                                 uint32_t *__restrict__ ofirst) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o = (uint32_t)(okeys[i].y >> kOidBit) & ((1u << kOidBit) - 1);
        if (o >= N) continue;
        if (i == 0 || ((uint32_t)(okeys[i - 1].y >> kOidBit) & ((1u << kOidBit) - 1)) != o)
            atomicMin(&ofirst[o], (uint32_t)i);
    }
}

__global__ void k_cmp_orun_index(const ulonglong2 *__restrict__ okeys, uint64_t n, uint32_t N,
                                 const uint16_t *__restrict__ sids, const uint32_t *__restrict__ ofirst,
                                 uint32_t *__restrict__ first, uint32_t *__restrict__ count) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x) {
        if (sids[o] != 1) continue;
        const uint32_t f = ofirst[o];
        uint32_t k = 0;
        if (f != 0xffffffffu)
            while (f + k < n && ((uint32_t)(okeys[f + k].y >> kOidBit) & ((1u << kOidBit) - 1)) == o) ++k;
        first[o] = k ? f : 0u;
        count[o] = k;
    }
}

__global__ void k_cmp_obitmap(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kBitBytes / 4; i += gridDim.x * blockDim.x)
        dst[i] |= src[i];
}

__global__ void k_cmp_sids_init(uint32_t N, const uint8_t *__restrict__ cls, uint16_t *__restrict__ sids) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < N; o += gridDim.x * blockDim.x) sids[o] = cls[o];
}

__global__ void k_cmp_ecs(uint32_t n, const unsigned long long *__restrict__ cstart, const uint32_t *__restrict__ escan,
                          uint32_t *__restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = escan[cstart[i]];
}

__global__ void k_cmp_iota(uint64_t n, uint32_t *__restrict__ perm, const unsigned long long *__restrict__ lo,
                           unsigned long long *__restrict__ keys) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        perm[i] = (uint32_t)i;
        keys[i] = lo[i];
    }
}

/* device scratch from the context's compaction pool, released on the stream
 * when the call returns (the pool keeps it mapped for the next merge) */
struct Scratch {
    cudaStream_t s;
    cudaMemPool_t pool;
    std::vector<void *> ptrs;
    cudaError_t e = cudaSuccess;
    Scratch(cudaStream_t st, cudaMemPool_t p) : s(st), pool(p) {}
    template <class T> T *get(size_t n) {
        void *p = nullptr;
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&p, (n ? n : 1) * sizeof(T), pool, s);
        if (e == cudaSuccess) ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    ~Scratch() {
        for (void *p : ptrs) cudaFreeAsync(p, s);
    }
};

} // namespace
} // namespace glint

using namespace glint;

extern "C" glint_status glint_store_compact(glint_ctx *c, uint32_t first, uint32_t count, uint32_t split_num,
                                            glint_compact_info *info) {
    if (!c || count == 0 || split_num == 0) return GLINT_ERR_INVALID_ARGUMENT;
    if ((uint64_t)first + count > c->ctbs.size()) {
        c->last_error = "compact: no such kept blocks";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    auto domain = [&](const std::string &why) {
        c->last_error = "compact: " + why;
        c->h_cnt->error_flags |= GLINT_EF_STORE_DOMAIN;
        return GLINT_ERR_UNSUPPORTED;
    };
    if (split_num > 255) return domain("split_num beyond the 16-bit sids (at most 255)");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    cudaError_t e = cudaStreamSynchronize(s);
    const uint32_t N = c->N, S2 = split_num * split_num, sn = split_num;
    auto cuda_fail = [&](cudaError_t err, const char *what) {
        c->last_error = std::string("compact: ") + what + ": " + cudaGetErrorString(err);
        return err == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    };
    if (e != cudaSuccess) return cuda_fail(e, "stream");
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        Events() {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
        }
        ~Events() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } ev;
    cudaEventRecord(ev.a, s);

    /* the source blocks and their CTFs' decode tables */
    std::vector<SrcBlock> hs(count);
    std::vector<std::vector<uint3>> toffs(count);
    uint64_t R = 0, O_src = 0, nf = 0, nd = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const StoreBlock &b = c->ctbs[first + i];
        std::vector<glint_ctf_meta> m(b.C);
        if (b.C && (e = cudaMemcpy(m.data(), b.ctfs, sizeof(glint_ctf_meta) * b.C, cudaMemcpyDefault)) !=
                       cudaSuccess)
            return cuda_fail(e, "source CTFs");
        toffs[i].resize(b.C ? b.C : 1);
        for (uint32_t j = 0; j < b.C; ++j) {
            if (m[j].low_x_bit > 24 || m[j].low_y_bit > 24 || m[j].edge_bit > 24)
                return domain("a source CTF's box bits beyond 24");
            toffs[i][j] = make_uint3((uint32_t)nf, (uint32_t)(nf + (1ull << m[j].low_x_bit)), (uint32_t)nd);
            nf += (1ull << m[j].low_x_bit) + (1ull << m[j].low_y_bit);
            nd += 1ull << m[j].edge_bit;
        }
        hs[i] = SrcBlock{b.keys, b.ctfs, b.key_index, b.byte_index, b.sids, nullptr, R, b.key_bytes, b.C, 0};
        R += b.kv;
        O_src += b.o_count;
    }
    if (R >= (1ull << 32) - 1 || O_src + R >= (1ull << 32) - 1) return domain("more than 2^32 keys");
    if (nf >= (1ull << 32) || nd >= (1ull << 32)) return domain("decode tables too large");
    if (!c->compact_pool) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = c->device;
        if ((e = cudaMemPoolCreate(&c->compact_pool, &props)) != cudaSuccess) {
            c->compact_pool = nullptr;
            return cuda_fail(e, "memory pool");
        }
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(c->compact_pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    Scratch sc(s, c->compact_pool);
    float *tf = sc.get<float>(nf);
    double *td = sc.get<double>(nd);
    for (uint32_t i = 0; i < count; ++i) {
        uint3 *t = sc.get<uint3>(toffs[i].size());
        if (sc.e != cudaSuccess) return cuda_fail(sc.e, "scratch");
        cudaMemcpyAsync(t, toffs[i].data(), sizeof(uint3) * toffs[i].size(), cudaMemcpyHostToDevice, s);
        hs[i].toff = t;
        if (hs[i].C) k_cmp_tables<<<hs[i].C, 256, 0, s>>>(hs[i].ctfs, t, tf, td);
    }
    SrcBlock *d_src = sc.get<SrcBlock>(count);
    unsigned long long *d_cnt = sc.get<unsigned long long>(kNumCounters);
    Rec *recs = sc.get<Rec>(R), *prec = sc.get<Rec>(R);
    unsigned long long *skey = sc.get<unsigned long long>(R), *skey2 = sc.get<unsigned long long>(R);
    uint32_t *sval = sc.get<uint32_t>(R), *sval2 = sc.get<uint32_t>(R);
    const uint64_t sort_n = std::max<uint64_t>(std::max<uint64_t>(R, N), O_src + R);
    void *rs_tmp = sc.get<uint8_t>(radix_tmp_bytes(sort_n));
    void *scan_tmp = sc.get<uint8_t>(scan_tmp_bytes(256 * ((sort_n + 1023) / 1024) + 1 + N + 1));
    uint32_t *rfirst = sc.get<uint32_t>(N), *rend = sc.get<uint32_t>(N), *nkeys = sc.get<uint32_t>(N);
    float4 *obox = sc.get<float4>(N);
    uint2 *ostart = sc.get<uint2>(N);
    uint8_t *cls = sc.get<uint8_t>(N);
    uint32_t *is2 = sc.get<uint32_t>(N + 1), *pos2 = sc.get<uint32_t>(N + 1);
    unsigned long long *xkey = sc.get<unsigned long long>(N), *ykey = sc.get<unsigned long long>(N);
    if (sc.e != cudaSuccess) return cuda_fail(sc.e, "scratch");
    cudaMemcpyAsync(d_src, hs.data(), sizeof(SrcBlock) * count, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * kNumCounters, s);
    cudaMemsetAsync(rfirst, 0, sizeof(uint32_t) * N, s);
    cudaMemsetAsync(rend, 0, sizeof(uint32_t) * N, s);

    /* parse and order the keys */
    if (R) k_cmp_parse<<<grid_for(R, 256), 256, 0, s>>>(d_src, count, R, N, tf, td, recs, skey, sval, d_cnt);
    if ((e = radix_sort_u64(skey, sval, skey2, sval2, R, 53, rs_tmp, scan_tmp, s)) != cudaSuccess)
        return cuda_fail(e, "key sort");
    unsigned long long hc[kNumCounters];
    if ((e = cudaMemcpyAsync(hc, d_cnt, sizeof(hc), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "parse");
    if (hc[kErrOid]) return domain("a key's object id is beyond num_objects");
    const uint64_t n_extra = hc[kExtraCount], R_ctf = R - n_extra;
    if (R) k_cmp_permute<<<grid_for(R, 256), 256, 0, s>>>(R, sval, recs, prec);
    if (R_ctf) k_cmp_runs<<<grid_for(R_ctf, 256), 256, 0, s>>>(skey, R_ctf, rfirst, rend);
    k_cmp_objects<<<grid_for(N, 256), 256, 0, s>>>(N, rfirst, rend, prec, d_src, count, nkeys, obox, ostart, cls,
                                                   is2, xkey, ykey);

    /* STR: the objects marked 2, by x middle */
    scan_u32(is2, pos2, N, scan_tmp, s);
    uint32_t S = 0, n0 = 0;
    if ((e = cudaMemcpyAsync(&S, pos2 + N, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&n0, nkeys, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "objects");
    if (S == 0) return domain("no object has a CTF key");
    const uint32_t split = S - 1, x_part = split / sn + 1, y_part = x_part / sn + 1;
    const int64_t last = (int64_t)split - (int64_t)x_part * (sn - 1) - (int64_t)y_part * (sn - 1);
    if (last < 0) return domain("too few objects for split_num (a partition size underflows)");
    unsigned long long *lk = sc.get<unsigned long long>(S), *lk2 = sc.get<unsigned long long>(S);
    uint32_t *lv = sc.get<uint32_t>(S), *lv2 = sc.get<uint32_t>(S), *yv = sc.get<uint32_t>(S);
    unsigned long long *yk = sc.get<unsigned long long>(S);
    unsigned long long *ck = sc.get<unsigned long long>(S);
    uint32_t *olist = sc.get<uint32_t>(S), *nl = sc.get<uint32_t>(S + 1), *escan = sc.get<uint32_t>(S + 1);
    uint32_t *posof = sc.get<uint32_t>(N), *ctf_of = sc.get<uint32_t>(N);
    uint16_t *nsids = sc.get<uint16_t>(N);
    if (sc.e != cudaSuccess) return cuda_fail(sc.e, "scratch");
    k_cmp_list2<<<grid_for(N, 256), 256, 0, s>>>(N, is2, pos2, xkey, lk, lv);
    if ((e = radix_sort_u64_varying(lk, lv, lk2, lv2, S, 32, rs_tmp, scan_tmp, s)) != cudaSuccess)
        return cuda_fail(e, "x sort");
    /* lv: the x order.  Inside each x part by y (stable), then by part */
    k_cmp_ykeys<<<grid_for(S, 256), 256, 0, s>>>(S, lv, ykey, yk, yv);
    if ((e = radix_sort_u64_varying(yk, yv, lk2, lv2, S, 32, rs_tmp, scan_tmp, s)) != cudaSuccess)
        return cuda_fail(e, "y sort");
    k_cmp_parts<<<grid_for(S, 256), 256, 0, s>>>(S, split, x_part, sn, yv, yk);
    if ((e = radix_sort_u64(yk, yv, lk2, lv2, S, 16, rs_tmp, scan_tmp, s)) != cudaSuccess)
        return cuda_fail(e, "part sort");
    /* sids: the class (0, 1, 2), then the CTF of every placed position; the
     * placed objects in (CTF, oid) order */
    k_cmp_sids_init<<<grid_for(N, 256), 256, 0, s>>>(N, cls, nsids);
    cudaMemsetAsync(ctf_of, 0xff, sizeof(uint32_t) * N, s);
    if (split) k_cmp_assign<<<grid_for(split, 256), 256, 0, s>>>(split, x_part, y_part, sn, yv, lv, nsids, ctf_of);
    k_cmp_placed<<<grid_for(N, 256), 256, 0, s>>>(N, ctf_of, is2);
    scan_u32(is2, pos2, N, scan_tmp, s);
    k_cmp_plist<<<grid_for(N, 256), 256, 0, s>>>(N, ctf_of, pos2, ck, olist);
    if ((e = radix_sort_u64(ck, olist, lk2, lv2, split, std::max(1, radix_bits_for(S2 - 1)), rs_tmp, scan_tmp, s)) !=
        cudaSuccess)
        return cuda_fail(e, "CTF sort");
    cudaMemsetAsync(posof, 0xff, sizeof(uint32_t) * N, s);
    if (split) k_cmp_listn<<<grid_for(split, 256), 256, 0, s>>>(split, olist, nkeys, nl, posof);
    scan_u32(nl, escan, split, scan_tmp, s);

    /* per CTF: its object-list size (merge_dump :908-911), the positions
     * that fill it, and the entries left to object 0 */
    std::vector<unsigned long long> h_cstart(S2 + 1, 0), h_pad(S2, 0);
    for (uint32_t cc = 0; cc < S2; ++cc) {
        const uint32_t xi = cc / sn, yi = cc % sn;
        const int64_t len = std::min<int64_t>(x_part, (int64_t)split - (int64_t)xi * x_part);
        const int64_t real = std::max<int64_t>(0, std::min<int64_t>(y_part, len - (int64_t)yi * y_part));
        const int64_t size = cc + 1 < S2 ? (int64_t)y_part : last;
        h_cstart[cc + 1] = h_cstart[cc] + (unsigned long long)real;
        h_pad[cc] = (unsigned long long)(size - real);
    }
    if (h_cstart[S2] != split) return domain("internal: CTF list sizes do not add up");
    unsigned long long *d_cstart = sc.get<unsigned long long>(S2 + 1), *d_pad = sc.get<unsigned long long>(S2);
    uint32_t *d_ecs = sc.get<uint32_t>(S2 + 1);
    float4 *d_lim = sc.get<float4>(S2);
    uint2 *d_slim = sc.get<uint2>(S2);
    if (sc.e != cudaSuccess) return cuda_fail(sc.e, "scratch");
    cudaMemcpyAsync(d_cstart, h_cstart.data(), sizeof(unsigned long long) * (S2 + 1), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_pad, h_pad.data(), sizeof(unsigned long long) * S2, cudaMemcpyHostToDevice, s);
    k_cmp_ecs<<<grid_for(S2 + 1, 256), 256, 0, s>>>(S2 + 1, d_cstart, escan, d_ecs);
    k_cmp_limits<<<S2, 256, 0, s>>>(d_cstart, olist, obox, ostart, d_pad, n0, d_lim, d_slim);
    std::vector<uint32_t> h_ecs(S2 + 1);
    std::vector<float4> h_lim(S2);
    std::vector<uint2> h_slim(S2);
    cudaMemcpyAsync(h_ecs.data(), d_ecs, sizeof(uint32_t) * (S2 + 1), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(h_lim.data(), d_lim, sizeof(float4) * S2, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(h_slim.data(), d_slim, sizeof(uint2) * S2, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "limits");

    /* the merged block's times (merge_dump :966-976): from the CTB records */
    uint32_t rec[4] = {1u << 30, 0, 1u << 30, 0}, ot[4] = {0, 0, 0, 0}, last_time = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const StoreBlock &b = c->ctbs[first + i];
        rec[0] = std::min(rec[0], b.rec_times[0]);
        rec[1] = std::max(rec[1], b.rec_times[1]);
        rec[2] = std::min(rec[2], b.rec_times[2]);
        rec[3] = std::max(rec[3], b.rec_times[3]);
        ot[0] = std::min(ot[0], b.o_times[0]);
        ot[1] = std::max(ot[1], b.o_times[1]);
        ot[2] = std::min(ot[2], b.o_times[2]);
        ot[3] = std::max(ot[3], b.o_times[3]);
        last_time = std::max(last_time, b.end_time_max);
    }
    /* CTF records, get_ctf_bits on the host */
    std::vector<glint_ctf_meta> metas(S2);
    std::vector<unsigned long long> h_ki(S2 + 1, 0), h_bi(S2 + 1, 0);
    for (uint32_t cc = 0; cc < S2; ++cc) {
        glint_ctf_meta &m = metas[cc];
        std::memset(&m, 0, sizeof(m));
        m.ctf_mbr[0] = h_lim[cc].x;
        m.ctf_mbr[1] = h_lim[cc].y;
        m.ctf_mbr[2] = h_lim[cc].z;
        m.ctf_mbr[3] = h_lim[cc].w;
        const uint64_t cap = h_pad[cc] * n0 + (h_ecs[cc + 1] - h_ecs[cc]);
        if (cap >= (1ull << 32)) return domain("a CTF of more than 2^32 keys");
        m.CTF_kv_capacity = (uint32_t)cap;
        m.start_time_min = h_slim[cc].x;
        m.start_time_max = h_slim[cc].y;
        m.end_time_min = rec[2];
        m.end_time_max = rec[3];
        if (!ctf_bits(m, c->mbr, N, c->cfg.max_meet_time))
            return domain("CTF " + std::to_string(cc) + " is outside get_ctf_bits' domain (an empty CTF?)");
        h_ki[cc + 1] = h_ki[cc] + cap;
        h_bi[cc + 1] = h_bi[cc] + cap * (m.key_bit / 8);
    }
    const uint64_t KV = h_ki[S2], KB = h_bi[S2];
    if (KV >= (1ull << 32)) return domain("more than 2^32 keys in the new block");
    const uint64_t O = O_src + n_extra;

    /* the new block */
    StoreBlock nb;
    cudaError_t ae = cudaSuccess;
    auto A = [&](void **p, size_t n) {
        if (ae == cudaSuccess) ae = cudaMalloc(p, n ? n : 1);
    };
    A((void **)&nb.keys, KB);
    A((void **)&nb.ctfs, sizeof(glint_ctf_meta) * S2);
    A((void **)&nb.key_index, sizeof(unsigned long long) * (S2 + 1));
    A((void **)&nb.byte_index, sizeof(unsigned long long) * (S2 + 1));
    A((void **)&nb.sids, sizeof(uint16_t) * N);
    A((void **)&nb.first, sizeof(uint32_t) * N);
    A((void **)&nb.count, sizeof(uint32_t) * N);
    A((void **)&nb.okeys, sizeof(ulonglong2) * O);
    A((void **)&nb.oboxes, sizeof(float4) * O);
    A((void **)&nb.bitmaps, (size_t)S2 * kBitBytes);
    A((void **)&nb.obitmap, kBitBytes);
    if (ae != cudaSuccess) {
        store_block_release(nb);
        return cuda_fail(ae, "new block");
    }
    cudaMemcpyAsync(nb.ctfs, metas.data(), sizeof(glint_ctf_meta) * S2, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(nb.key_index, h_ki.data(), sizeof(unsigned long long) * (S2 + 1), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(nb.byte_index, h_bi.data(), sizeof(unsigned long long) * (S2 + 1), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(nb.sids, nsids, sizeof(uint16_t) * N, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(nb.bitmaps, 0, (size_t)S2 * kBitBytes, s);
    cudaMemsetAsync(nb.obitmap, 0, kBitBytes, s);

    /* bitmaps and packed keys: every placed object's records, then object
     * 0's repeats */
    std::vector<unsigned long long> h_padk(S2 + 1, 0);
    for (uint32_t cc = 0; cc < S2; ++cc) h_padk[cc + 1] = h_padk[cc] + h_pad[cc] * n0;
    unsigned long long *d_padk = sc.get<unsigned long long>(S2 + 1), *obase = sc.get<unsigned long long>(N);
    if (sc.e != cudaSuccess) {
        store_block_release(nb);
        return cuda_fail(sc.e, "scratch");
    }
    cudaMemcpyAsync(d_padk, h_padk.data(), sizeof(unsigned long long) * (S2 + 1), cudaMemcpyHostToDevice, s);
    k_cmp_index<<<grid_for(N, 256), 256, 0, s>>>(N, nsids, nkeys, posof, d_cstart, nb.key_index, d_pad, escan, olist,
                                                 S2, n0, nb.first, nb.count, obase);
    PackArgs pa;
    pa.ctfs = nb.ctfs;
    pa.key_index = nb.key_index;
    pa.byte_index = nb.byte_index;
    pa.cstart = d_cstart;
    pa.pad = d_pad;
    pa.padk = d_padk;
    pa.escan = escan;
    pa.posof = posof;
    pa.rfirst = rfirst;
    pa.ctf_of = ctf_of;
    pa.obase = obase;
    pa.prec = prec;
    pa.out = nb.keys;
    pa.bits = reinterpret_cast<uint32_t *>(nb.bitmaps);
    pa.counters = d_cnt;
    pa.C = S2;
    pa.n0 = n0;
    /* the output-order records reuse the parsed records' buffer when they fit */
    Rec *ordered = KV <= R ? recs : sc.get<Rec>(KV);
    if (sc.e != cudaSuccess) {
        store_block_release(nb);
        return cuda_fail(sc.e, "scratch");
    }
    pa.n = R_ctf;
    if (R_ctf) k_cmp_place<<<grid_for(R_ctf, 256), 256, 0, s>>>(pa, ordered);
    pa.n = h_padk[S2];
    if (pa.n) k_cmp_place_pad<<<grid_for(pa.n, 256), 256, 0, s>>>(pa, ordered);
    /* the pack's chunks: (CTF, first key) for every kPackChunk keys of every CTF */
    std::vector<uint2> h_chunks;
    for (uint32_t cc = 0; cc < S2; ++cc)
        for (uint64_t k = 0; k < h_ki[cc + 1] - h_ki[cc]; k += kPackChunk) h_chunks.push_back(make_uint2(cc, (uint32_t)k));
    uint2 *d_chunks = sc.get<uint2>(h_chunks.size());
    if (sc.e != cudaSuccess) {
        store_block_release(nb);
        return cuda_fail(sc.e, "scratch");
    }
    if (!h_chunks.empty()) {
        cudaMemcpyAsync(d_chunks, h_chunks.data(), sizeof(uint2) * h_chunks.size(), cudaMemcpyHostToDevice, s);
        k_cmp_pack<<<(unsigned)h_chunks.size(), 256, 0, s>>>(pa, ordered, d_chunks);
    }

    /* the oversize buffers (merge_dump :1099-1127): the smallest head key is
     * taken each time, ties to the earlier buffer, the extra list last.  For
     * buffers in key order that is a stable sort of their concatenation; and
     * while every source key carries sid bits, every extra key (without them)
     * is smaller, so the extra list leads in its own order */
    if (O) {
        for (uint32_t i = 0; i < count; ++i) {
            const StoreBlock &b = c->ctbs[first + i];
            if (b.o_count) k_cmp_ocheck<<<grid_for(b.o_count, 256), 256, 0, s>>>(b.okeys, b.o_count, d_cnt);
        }
        if (n_extra > 1) k_cmp_xcheck<<<grid_for(n_extra, 256), 256, 0, s>>>(prec, R_ctf, n_extra, d_cnt);
        if ((e = cudaMemcpyAsync(hc, d_cnt, sizeof(hc), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess) {
            store_block_release(nb);
            return cuda_fail(e, "oversize check");
        }
        if (hc[kErrOrder]) {
            store_block_release(nb);
            return domain("a source oversize buffer is out of key order");
        }
        const bool extra_first = n_extra && hc[kNoSid] == 0;
        if (n_extra && !extra_first && hc[kExtraOrder]) {
            store_block_release(nb);
            return domain("the extra oversize list would interleave out of key order");
        }
        unsigned long long *olo = sc.get<unsigned long long>(O), *ohi = sc.get<unsigned long long>(O);
        unsigned long long *okk = sc.get<unsigned long long>(O), *okk2 = sc.get<unsigned long long>(O);
        uint32_t *operm = sc.get<uint32_t>(O), *operm2 = sc.get<uint32_t>(O), *ofirst = sc.get<uint32_t>(N);
        float4 *obx = sc.get<float4>(O);
        if (sc.e != cudaSuccess) {
            store_block_release(nb);
            return cuda_fail(sc.e, "scratch");
        }
        uint64_t at = 0;
        if (extra_first) {
            k_cmp_ocat<<<grid_for(n_extra, 256), 256, 0, s>>>(nullptr, nullptr, 0, prec, R_ctf, n_extra, olo,
                                                              ohi, obx, 0);
            at = n_extra;
        }
        for (uint32_t i = 0; i < count; ++i) {
            const StoreBlock &b = c->ctbs[first + i];
            const uint64_t ne = (!extra_first && i + 1 == count) ? n_extra : 0;
            if (b.o_count + ne)
                k_cmp_ocat<<<grid_for(b.o_count + ne, 256), 256, 0, s>>>(b.okeys, b.oboxes, b.o_count, prec,
                                                                         R_ctf, ne, olo, ohi, obx, at);
            at += b.o_count + ne;
        }
        /* the sorted range: everything but a leading extra list */
        const uint64_t off = extra_first ? n_extra : 0, ns = O - off;
        k_cmp_iota<<<grid_for(O, 256), 256, 0, s>>>(O, operm, olo, okk);
        if ((e = radix_sort_u64(okk + off, operm + off, okk2, operm2, ns, 64, rs_tmp, scan_tmp, s)) != cudaSuccess) {
            store_block_release(nb);
            return cuda_fail(e, "oversize sort");
        }
        k_cmp_gather_hi<<<grid_for(ns, 256), 256, 0, s>>>(ns, operm + off, ohi, okk + off);
        if ((e = radix_sort_u64(okk + off, operm + off, okk2, operm2, ns, 64, rs_tmp, scan_tmp, s)) != cudaSuccess) {
            store_block_release(nb);
            return cuda_fail(e, "oversize sort");
        }
        k_cmp_ogather<<<grid_for(O, 256), 256, 0, s>>>(O, operm, olo, ohi, obx, nb.okeys, nb.oboxes);
        cudaMemsetAsync(ofirst, 0xff, sizeof(uint32_t) * N, s);
        k_cmp_orun_first<<<grid_for(O, 256), 256, 0, s>>>(nb.okeys, O, N, ofirst);
        k_cmp_orun_index<<<grid_for(N, 256), 256, 0, s>>>(nb.okeys, O, N, nsids, ofirst, nb.first, nb.count);
    }
    for (uint32_t i = 0; i < count; ++i)
        k_cmp_obitmap<<<2, 1024, 0, s>>>(reinterpret_cast<const uint32_t *>(c->ctbs[first + i].obitmap),
                                         reinterpret_cast<uint32_t *>(nb.obitmap));
    cudaEventRecord(ev.b, s);
    if ((e = cudaMemcpyAsync(hc, d_cnt, sizeof(hc), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
        store_block_release(nb);
        return cuda_fail(e, "merge");
    }
    if (hc[kErrCells]) {
        store_block_release(nb);
        return domain("a key box covers more bitmap cells than supported");
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev.a, ev.b);

    std::vector<uint16_t> hsids(N);
    if ((e = cudaMemcpy(hsids.data(), nsids, sizeof(uint16_t) * N, cudaMemcpyDeviceToHost)) != cudaSuccess) {
        store_block_release(nb);
        return cuda_fail(e, "sids");
    }
    nb.kv = KV;
    nb.o_count = O;
    nb.key_bytes = KB;
    nb.end_time_min = rec[2];
    nb.end_time_max = last_time;
    nb.C = S2;
    std::memcpy(nb.o_times, ot, sizeof(ot));
    std::memcpy(nb.rec_times, rec, sizeof(rec));
    nb.sid_count = split;
    for (uint32_t o = 0; o < N; ++o) nb.oversize_oid_count += hsids[o] == 1;
    nb.start_min = c->ctbs[first].start_min;
    nb.spans_known = true;
    for (uint32_t i = 0; i < count; ++i) {
        nb.start_min = std::min(nb.start_min, c->ctbs[first + i].start_min);
        nb.spans_known = nb.spans_known && c->ctbs[first + i].spans_known &&
                         c->ctbs[first + i].end_time_max <= last_time;
    }
    /* the new block takes the merged blocks' place (servers read the kept
     * blocks from their own streams) */
    cudaDeviceSynchronize();
    for (uint32_t i = 0; i < count; ++i) store_block_release(c->ctbs[first + i]);
    c->ctbs.erase(c->ctbs.begin() + first, c->ctbs.begin() + first + count);
    c->ctbs.insert(c->ctbs.begin() + first, nb);
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->CTF_count = S2;
        info->blocks = count;
        info->kv_count = KV;
        info->key_bytes = KB;
        uint64_t padded = 0;
        for (uint32_t cc = 0; cc < S2; ++cc) padded += h_pad[cc];
        info->padding = padded;
        info->oversize_kv_count = (uint32_t)O;
        info->sid_count = split;
        info->x_part = x_part;
        info->y_part = y_part;
        info->ms = ms;
    }
    return GLINT_OK;
}
