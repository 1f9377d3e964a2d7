/*
 * glint_flush_oracle.c -- CPU restatement of the GPU path's key generation and
 * of the flush of finished meetings into the sorted key-value + bitmap store.
 *
 * TEST INFRASTRUCTURE: used only by tests/ and bench.py's CPU legs.
 *
 * The reference produces the store only on its GPU path:
 *   key generation   cuda_identify_meetings (cuda/geometry.cu:665-734)
 *   flush            process_with_gpu "4.5 cuda sort" (cuda/geometry.cu:1752-2135)
 *                    with set_oid, narrow_xy_to_y, make_sid, write_sid_in_key,
 *                    get_CTF_capacity, cuda_get_limit, get_o_limit,
 *                    cuda_write_o_bitmap, cuda_write_bitmap, write_key_and_mbr
 *                    (cuda/geometry.cu:739-1107), serialize_mbr (:162-174),
 *                    CTF::get_ctf_bits / eight_parallel (tracing/step_merge.cpp:132-186)
 * and the host-side window update of straight_dump (tracing/process.cpp:271,549).
 * Each step is restated in the reference's arithmetic (float where it uses
 * float, double where it promotes to double) with the GPU's conversion rules:
 * float/double -> unsigned conversions saturate (negative and NaN -> 0).
 *
 * Two of the reference's block reductions (cuda_get_limit, get_o_limit) fold
 * shared memory down to 64 partial results and then reduce only the first 32
 * with warp shuffles; partial results 32..63 are never combined.  With
 * 1024-thread blocks striding over the keys, a key at offset o from the start
 * of its range therefore contributes only when o mod 64 < 32.  That is
 * restated here (limit_counts) because the CTF boxes it yields decide the bit
 * widths, the bitmaps and the packed keys.
 *
 * Sorting: the reference sorts with thrust (radix sort, stable for primitive
 * keys).  The STR sorts here are stable; the key sorts are total (keys are
 * unique), so the order is fully determined.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "glint_oracle.h"

typedef unsigned __int128 u128;

#define FO_OID_BIT 26          /* util/util.h:49 */
#define FO_DURATION_BIT 32     /* util/util.h:51 */
#define FO_END_BIT 32          /* util/util.h:52 */
#define FO_BITMAP_EDGE 256     /* DEFAULT_bitmap_edge, util/util.h:47 */

struct go_store {
    go_store_config cfg;
    uint32_t end_time_min;

    /* key state (accumulated by go_store_add_meetings) */
    u128 *keys;
    float *boxes;               /* [kv_capacity][4] low0 low1 high0 high1 */
    uint64_t kv_count;
    uint32_t *same_pid_count;
    uint32_t *o_boxs;           /* [N][4] uint_box low0 low1 high0 high1 */
    uint16_t *sids;
    uint32_t sid_count;
    uint32_t oversize_oid_count;
    uint32_t dropped;           /* meetings outside the map box (not keyed) */
    int overflow;

    /* result of the last flush */
    int have_result;
    go_store_info info;
    uint8_t *ctf_keys;          /* packed, kv_capacity * 16 bytes */
    uint16_t *out_sids;
    uint32_t *ctf_capacity;
    go_ctf_meta *ctfs;
    uint8_t *bitmaps;           /* CTF_count * bit_count / 8 */
    u128 *o_keys;
    float *o_boxes;
    uint8_t *o_bitmap;          /* bit_count / 8 */
};

/* ---- helpers in the reference's arithmetic ---- */

/* float_to_uint (cuda/cuda_util.cuh:116-120) */
static uint32_t f2u_coord(float xy) {
    volatile float a = xy + 180;
    volatile float b = a * 100000;
    return (uint32_t)b;
}
/* uint_to_float (cuda/cuda_util.cuh:122-126) */
static float u2f_coord(uint32_t f) {
    volatile float a = (float)f / 100000;
    volatile float b = a - 180;
    return b;
}
/* GPU float -> unsigned conversions saturate */
static uint32_t sat_u32_f(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)v;
}
static uint32_t sat_u32_d(double v) {
    if (!(v > 0.0)) return 0;
    if (v >= 4294967296.0) return 0xffffffffu;
    return (uint32_t)v;
}
static uint64_t sat_u64_f(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 18446744073709551616.0f) return ~0ull;
    return (uint64_t)v;
}
/* min_bits_to_store (util/util.h:527-533): floor(log2(v)) + 1, 1 for 0 */
static uint32_t min_bits(uint32_t v) {
    if (v == 0) return 1;
    uint32_t b = 0;
    while (v) { ++b; v >>= 1; }
    return b;
}
static uint32_t key_oid(u128 k) { return (uint32_t)((k >> (FO_OID_BIT + FO_DURATION_BIT + FO_END_BIT)) & ((1u << FO_OID_BIT) - 1)); }
static uint32_t key_duration(u128 k) { return (uint32_t)((k >> FO_END_BIT) & 0xffffffffu); }
static uint32_t key_end(u128 k) { return (uint32_t)(k & 0xffffffffu); }

go_store *go_store_create(const go_store_config *cfg) {
    go_store *s = (go_store *)calloc(1, sizeof(go_store));
    s->cfg = *cfg;
    const uint32_t N = cfg->num_objects;
    s->end_time_min = cfg->first_end_time_min;
    s->keys = (u128 *)calloc(cfg->kv_capacity ? cfg->kv_capacity : 1, sizeof(u128));
    s->boxes = (float *)calloc((cfg->kv_capacity ? cfg->kv_capacity : 1) * 4, sizeof(float));
    s->same_pid_count = (uint32_t *)calloc(N, sizeof(uint32_t));
    s->o_boxs = (uint32_t *)calloc((size_t)N * 4, sizeof(uint32_t));
    s->sids = (uint16_t *)calloc(N, sizeof(uint16_t));
    /* cuda_init_o_boxs (cuda/geometry.cu:1254-1263) */
    for (uint32_t i = 0; i < N; ++i) {
        s->o_boxs[4 * i + 0] = 100000000;
        s->o_boxs[4 * i + 1] = 100000000;
        s->o_boxs[4 * i + 2] = 0;
        s->o_boxs[4 * i + 3] = 0;
    }
    const size_t bit_bytes = FO_BITMAP_EDGE * FO_BITMAP_EDGE / 8;
    s->ctf_keys = (uint8_t *)calloc((cfg->kv_capacity ? cfg->kv_capacity : 1) * 16, 1);
    s->out_sids = (uint16_t *)calloc(N, sizeof(uint16_t));
    s->ctf_capacity = (uint32_t *)calloc(cfg->CTF_count, sizeof(uint32_t));
    s->ctfs = (go_ctf_meta *)calloc(cfg->CTF_count, sizeof(go_ctf_meta));
    s->bitmaps = (uint8_t *)calloc((size_t)cfg->CTF_count * bit_bytes, 1);
    s->o_keys = (u128 *)calloc(cfg->kv_capacity ? cfg->kv_capacity : 1, sizeof(u128));
    s->o_boxes = (float *)calloc((cfg->kv_capacity ? cfg->kv_capacity : 1) * 4, sizeof(float));
    s->o_bitmap = (uint8_t *)calloc(bit_bytes, 1);
    return s;
}

void go_store_destroy(go_store *s) {
    if (!s) return;
    free(s->keys); free(s->boxes); free(s->same_pid_count); free(s->o_boxs); free(s->sids);
    free(s->ctf_keys); free(s->out_sids); free(s->ctf_capacity); free(s->ctfs); free(s->bitmaps);
    free(s->o_keys); free(s->o_boxes); free(s->o_bitmap);
    free(s);
}

/* cuda_identify_meetings, the report branch (cuda/geometry.cu:665-734), for
 * meetings (pid1 < pid2, start, end, f32 box) reported by one step */
void go_store_add_meetings(go_store *s, const go_meeting_rec *m, uint64_t n) {
    const double *mb = s->cfg.mbr;
    for (uint64_t i = 0; i < n; ++i) {
        const float *b = m[i].mbr;
        /* box_contain(&bench->mbr, &meeting.mbr) (cuda/geometry.cu:53-58) */
        if (!((double)b[0] >= mb[0] && (double)b[2] <= mb[2] && (double)b[1] >= mb[1] && (double)b[3] <= mb[3])) {
            s->dropped++;
            continue;
        }
        const uint32_t duration = m[i].end - m[i].start;
        uint32_t pid = m[i].pid1, target = m[i].pid2;
        if (duration > s->cfg.max_meet_time) {
            s->oversize_oid_count++;
            s->sids[pid] = 1;
            s->sids[target] = 1;
        }
        if (s->kv_count + 2 > s->cfg.kv_capacity) {
            s->overflow = 1;
            continue;
        }
        uint64_t idx = s->kv_count;
        s->kv_count += 2;
        for (int k = 0; k < 2; ++k) {
            if (k == 1) {
                ++idx;
                const uint32_t t = pid;
                pid = target;
                target = t;
            }
            s->keys[idx] = ((u128)pid << (FO_OID_BIT + FO_DURATION_BIT + FO_END_BIT)) +
                           ((u128)target << (FO_DURATION_BIT + FO_END_BIT)) +
                           ((u128)(m[i].end - m[i].start) << FO_END_BIT) + (u128)(uint32_t)(m[i].end - s->end_time_min);
            memcpy(s->boxes + 4 * idx, b, 4 * sizeof(float));
            if (s->same_pid_count[pid]++ == 0) s->sid_count++;
            uint32_t *o = s->o_boxs + 4 * (size_t)pid;
            const uint32_t l0 = f2u_coord(b[0]), h0 = f2u_coord(b[2]), l1 = f2u_coord(b[1]), h1 = f2u_coord(b[3]);
            if (l0 < o[0]) o[0] = l0;
            if (h0 > o[2]) o[2] = h0;
            if (l1 < o[1]) o[1] = l1;
            if (h1 > o[3]) o[3] = h1;
        }
    }
}

uint64_t go_store_kv_count(const go_store *s) { return s->kv_count; }

/* ---- sorting helpers ---- */
static const u128 *g_sort_keys;
static int cmp_idx_key(const void *a, const void *b) {
    const u128 x = g_sort_keys[*(const uint64_t *)a], y = g_sort_keys[*(const uint64_t *)b];
    return x < y ? -1 : x > y ? 1 : 0;
}
/* sorts keys[lo, hi) with their boxes by the full 128-bit key */
static void sort_keys_boxes(u128 *keys, float *boxes, uint64_t lo, uint64_t hi) {
    const uint64_t n = hi - lo;
    if (n < 2) return;
    uint64_t *idx = (uint64_t *)malloc(n * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; ++i) idx[i] = lo + i;
    g_sort_keys = keys;
    qsort(idx, n, sizeof(uint64_t), cmp_idx_key);
    u128 *tk = (u128 *)malloc(n * sizeof(u128));
    float *tb = (float *)malloc(n * 4 * sizeof(float));
    for (uint64_t i = 0; i < n; ++i) {
        tk[i] = keys[idx[i]];
        memcpy(tb + 4 * i, boxes + 4 * idx[i], 4 * sizeof(float));
    }
    memcpy(keys + lo, tk, n * sizeof(u128));
    memcpy(boxes + 4 * lo, tb, n * 4 * sizeof(float));
    free(tk); free(tb); free(idx);
}
/* stable sort of (u64 key, u32 value) pairs on [lo, hi) */
typedef struct { uint64_t k; uint32_t v; uint32_t pos; } kv64;
static int cmp_kv64(const void *a, const void *b) {
    const kv64 *x = (const kv64 *)a, *y = (const kv64 *)b;
    if (x->k != y->k) return x->k < y->k ? -1 : 1;
    return x->pos < y->pos ? -1 : x->pos > y->pos ? 1 : 0;
}
static void stable_sort_by_key(uint64_t *k, uint32_t *v, uint64_t lo, uint64_t hi) {
    if (hi <= lo + 1) return;
    const uint64_t n = hi - lo;
    kv64 *t = (kv64 *)malloc(n * sizeof(kv64));
    for (uint64_t i = 0; i < n; ++i) { t[i].k = k[lo + i]; t[i].v = v[lo + i]; t[i].pos = (uint32_t)i; }
    qsort(t, n, sizeof(kv64), cmp_kv64);
    for (uint64_t i = 0; i < n; ++i) { k[lo + i] = t[i].k; v[lo + i] = t[i].v; }
    free(t);
}

/* the reductions of cuda_get_limit / get_o_limit over keys[lo, lo + n):
 * offsets o with o mod 64 >= 32 are lost (see the header) */
static void limit_counts(const go_store *s, const u128 *keys, const float *boxes, uint64_t lo, uint64_t n,
                         int with_box, float box[4], uint32_t *start_min, uint32_t *start_max) {
    float l0 = 100000.0f, l1 = 100000.0f, h0 = -100000.0f, h1 = -100000.0f;
    int32_t smin = 1 << 30, smax = 0;
    for (uint64_t o = 0; o < n; ++o) {
        if ((o & 63) >= 32) continue;
        const uint64_t kid = lo + o;
        if (with_box) {
            const float *b = boxes + 4 * kid;
            l0 = fminf(l0, b[0]);
            l1 = fminf(l1, b[1]);
            h0 = fmaxf(h0, b[2]);
            h1 = fmaxf(h1, b[3]);
        }
        const uint32_t duration = key_duration(keys[kid]);
        const uint32_t end = key_end(keys[kid]) + s->end_time_min;
        const uint32_t st = end - duration;
        if ((int32_t)st < smin) smin = (int32_t)st;
        if ((int32_t)st > smax) smax = (int32_t)st;
    }
    if (with_box) { box[0] = l0; box[1] = l1; box[2] = h0; box[3] = h1; }
    *start_min = (uint32_t)smin;
    *start_max = (uint32_t)smax;
}

/* CTF::get_ctf_bits + eight_parallel (tracing/step_merge.cpp:132-186);
 * returns 0 where the reference's asserts would fire */
static int ctf_bits(go_ctf_meta *c, const double *map, const go_store_config *cfg) {
    c->id_bit = (uint16_t)min_bits(cfg->num_objects);
    c->duration_bit = (uint16_t)min_bits(cfg->max_meet_time - 1);
    c->end_bit = c->duration_bit;
    volatile double map_x_grid_length = (map[2] - map[0]) / 3000;
    volatile double map_y_grid_length = (map[3] - map[1]) / 4200;
    volatile double gx = ((double)c->ctf_mbr[2] - (double)c->ctf_mbr[0]) / map_x_grid_length;
    volatile double gy = ((double)c->ctf_mbr[3] - (double)c->ctf_mbr[1]) / map_y_grid_length;
    if (!(gx >= 0.0) || !(gy >= 0.0)) return 0; /* an empty CTF: out of the reference's domain */
    const uint32_t low_x_grid = (uint32_t)gx, low_y_grid = (uint32_t)gy;
    c->low_x_bit = (uint16_t)min_bits((low_x_grid > 1 ? low_x_grid : 1) - 1);
    c->low_y_bit = (uint16_t)min_bits((low_y_grid > 1 ? low_y_grid : 1) - 1);
    c->edge_bit = c->low_x_bit > c->low_y_bit ? c->low_x_bit : c->low_y_bit;
    c->mbr_bit = (uint16_t)(c->low_x_bit + c->low_y_bit + 2 * c->edge_bit);
    if (c->mbr_bit > 64) return 0;
    const uint32_t temp_bit = c->id_bit * 2u + c->duration_bit + c->end_bit + c->mbr_bit;
    if (temp_bit > 128) return 0;
    c->key_bit = (uint16_t)(temp_bit / 8 * 8);
    if (c->key_bit < temp_bit) c->key_bit += 8;
    volatile double wx = ((double)c->ctf_mbr[2] - (double)c->ctf_mbr[0]) / (map[2] - map[0]) * 300;
    volatile double wy = ((double)c->ctf_mbr[3] - (double)c->ctf_mbr[1]) / (map[3] - map[1]) * 420;
    const int old_width_grid = (int)wx, old_high_grid = (int)wy;
    int xg = old_width_grid + 1 > 32 ? old_width_grid + 1 : 32;
    int yg = old_high_grid + 1 > 32 ? old_high_grid + 1 : 32;
    if (xg >= 256 || yg >= 256) {
        xg = old_width_grid + 1 < 255 ? old_width_grid + 1 : 255;
        yg = old_high_grid + 1 < 255 ? old_high_grid + 1 : 255;
    }
    c->x_grid = (uint16_t)xg;
    c->y_grid = (uint16_t)yg;
    c->ctf_bitmap_size = (uint32_t)(xg * yg + 7) / 8;
    return 1;
}

/* serialize_mbr for f_box (cuda/geometry.cu:162-174), GPU conversion rules */
static uint64_t serialize_box(const float *b, const go_ctf_meta *c) {
    const float *m = c->ctf_mbr;
    volatile float ex = m[2] - m[0], ey = m[3] - m[1];
    const float longer_edge = ex > ey ? ex : ey;
    volatile float t0 = (b[0] - m[0]) / ex * (float)((1ull << c->low_x_bit) - 1);
    volatile float t1 = (b[1] - m[1]) / ey * (float)((1ull << c->low_y_bit) - 1);
    volatile float tx = (b[2] - b[0]) / longer_edge * (float)((1ull << c->edge_bit) - 1);
    volatile float ty = (b[3] - b[1]) / longer_edge * (float)((1ull << c->edge_bit) - 1);
    const uint64_t low0 = sat_u64_f(t0), low1 = sat_u64_f(t1), x = sat_u64_f(tx), y = sat_u64_f(ty);
    return (low0 << (c->low_y_bit + c->edge_bit + c->edge_bit)) + (low1 << (c->edge_bit + c->edge_bit)) +
           (x << c->edge_bit) + y;
}

static void set_bit(uint8_t *bits, uint64_t nbits, uint64_t pos, uint64_t *outside) {
    if (pos < nbits) bits[pos >> 3] |= (uint8_t)(1u << (pos & 7));
    else if (outside) ++*outside;
}

int go_store_flush(go_store *s, uint32_t cur_time, go_store_info *out) {
    const go_store_config *cfg = &s->cfg;
    const uint32_t N = cfg->num_objects, C = cfg->CTF_count, split = cfg->split_num;
    const uint64_t bit_count = FO_BITMAP_EDGE * FO_BITMAP_EDGE;
    const double *map = cfg->mbr;
    memset(&s->info, 0, sizeof(s->info));
    if (s->overflow) return -1;

    uint32_t *oids = (uint32_t *)malloc(sizeof(uint32_t) * (N ? N : 1));
    uint64_t *mid_xys = (uint64_t *)calloc(N ? N : 1, sizeof(uint64_t));
    /* set_oid (cuda/geometry.cu:739-769) */
    for (uint32_t id = 0; id < N; ++id) {
        oids[id] = id;
        if (s->same_pid_count[id] >= 1) {
            const uint32_t *o = s->o_boxs + 4 * (size_t)id;
            const float low0 = u2f_coord(o[0]), high0 = u2f_coord(o[2]);
            const float low1 = u2f_coord(o[1]), high1 = u2f_coord(o[3]);
            volatile float dy = high1 - low1, dx = high0 - low0;
            volatile float area = dy * dx;
            if ((double)area > cfg->dProbFalse) {
                s->oversize_oid_count++;
                s->sids[id] = 1;
                continue;
            }
            const uint32_t ave_mid0 = o[0] / 2 + o[2] / 2;
            const uint32_t ave_mid1 = o[3] / 2 + o[3] / 2; /* high[1] twice, as the reference */
            mid_xys[id] = ((uint64_t)ave_mid0 << 32) + (uint64_t)ave_mid1;
        }
    }
    /* partition: keys whose object is not oversize first (cuda/geometry.cu:1784-1797) */
    const uint64_t old_kv = s->kv_count;
    u128 *k2 = (u128 *)malloc(sizeof(u128) * (old_kv ? old_kv : 1));
    float *b2 = (float *)malloc(sizeof(float) * 4 * (old_kv ? old_kv : 1));
    uint64_t main_n = 0;
    for (int pass = 0; pass < 2; ++pass)
        for (uint64_t i = 0; i < old_kv; ++i) {
            const int over = s->sids[key_oid(s->keys[i])] == 1;
            if (over != pass) continue;
            k2[main_n] = s->keys[i];
            memcpy(b2 + 4 * main_n, s->boxes + 4 * i, 4 * sizeof(float));
            ++main_n;
        }
    main_n = 0;
    for (uint64_t i = 0; i < old_kv; ++i)
        if (s->sids[key_oid(s->keys[i])] != 1) ++main_n;
    memcpy(s->keys, k2, sizeof(u128) * old_kv);
    memcpy(s->boxes, b2, sizeof(float) * 4 * old_kv);
    free(k2); free(b2);
    const uint64_t kv = main_n, o_n = old_kv - main_n;
    /* oversize buffer: sorted keys, get_o_limit, cuda_write_o_bitmap (:1803-1836, 909-1000) */
    sort_keys_boxes(s->keys, s->boxes, kv, old_kv);
    uint32_t o_smin, o_smax;
    limit_counts(s, s->keys, s->boxes, kv, o_n, 0, NULL, &o_smin, &o_smax);
    /* the oversize bitmap is drawn into the first CTF bitmap's space of the
     * bitmap array, copied out, and only those bit_count bits are cleared:
     * bits past them stay set in the following CTFs' bitmaps */
    const uint64_t total_bits = (uint64_t)C * bit_count;
    memset(s->bitmaps, 0, total_bits / 8);
    memset(s->o_bitmap, 0, bit_count / 8);
    uint64_t outside = 0;
    for (uint64_t i = 0; i < o_n; ++i) {
        const float *b = s->boxes + 4 * (kv + i);
        const uint32_t l0 = sat_u32_d(((double)b[0] - map[0]) / (map[2] - map[0]) * FO_BITMAP_EDGE);
        const uint32_t l1 = sat_u32_d(((double)b[1] - map[1]) / (map[3] - map[1]) * FO_BITMAP_EDGE);
        const uint32_t h0 = sat_u32_d(((double)b[2] - map[0]) / (map[2] - map[0]) * FO_BITMAP_EDGE);
        const uint32_t h1 = sat_u32_d(((double)b[3] - map[1]) / (map[3] - map[1]) * FO_BITMAP_EDGE);
        for (uint64_t x = l0; x <= h0 && x < total_bits; ++x)
            for (uint64_t y = l1; y <= h1 && x + y * FO_BITMAP_EDGE < total_bits; ++y) {
                const uint64_t pos = x + y * FO_BITMAP_EDGE;
                if (pos < bit_count) set_bit(s->o_bitmap, bit_count, pos, NULL);
                else set_bit(s->bitmaps, total_bits, pos, &outside);
            }
    }
    for (uint64_t i = 0; i < o_n; ++i) {
        s->o_keys[i] = s->keys[kv + i];
        memcpy(s->o_boxes + 4 * i, s->boxes + 4 * (kv + i), 4 * sizeof(float));
    }
    /* STR (cuda/geometry.cu:1862-1899) */
    stable_sort_by_key(mid_xys, oids, 0, N);
    const uint32_t zero_one = (N - s->sid_count) + s->oversize_oid_count;
    for (uint32_t id = zero_one; id < N; ++id) mid_xys[id] &= 0xffffffffull; /* narrow_xy_to_y */
    const uint32_t M = s->sid_count - s->oversize_oid_count;
    const uint32_t x_part = M / split + 1;
    for (uint32_t i = 0; i < split; ++i) {
        uint64_t lo = (uint64_t)zero_one + (uint64_t)x_part * i;
        uint64_t hi = i + 1 < split ? (uint64_t)zero_one + (uint64_t)x_part * (i + 1) : N;
        if (hi > N) hi = N;
        if (lo < hi) stable_sort_by_key(mid_xys, oids, lo, hi);
    }
    /* make_sid (cuda/geometry.cu:780-796) */
    const uint32_t part_key = x_part / split + 1;
    for (uint32_t id = zero_one; id < N; ++id) {
        const uint32_t xi = (id - zero_one) / x_part;
        const uint32_t yi = (id - zero_one - xi * x_part) / part_key;
        s->sids[oids[id]] = (uint16_t)(xi * split + yi + 2);
    }
    /* write_sid_in_key (:798-806) and the sort of the CTF keys (:1909) */
    const u128 low_mask = ((u128)1 << (FO_OID_BIT * 2 + FO_DURATION_BIT + FO_END_BIT)) - 1;
    for (uint64_t k = 0; k < kv; ++k)
        s->keys[k] = (s->keys[k] & low_mask) + ((u128)s->sids[key_oid(s->keys[k])] << (FO_OID_BIT * 2 + FO_DURATION_BIT + FO_END_BIT));
    sort_keys_boxes(s->keys, s->boxes, 0, kv);
    /* get_CTF_capacity (:808-818) */
    memset(s->ctf_capacity, 0, sizeof(uint32_t) * C);
    for (uint32_t id = zero_one; id < N; ++id) {
        const uint32_t oid = oids[id];
        const uint32_t ctf = (uint32_t)s->sids[oid] - 2;
        if (ctf < C) s->ctf_capacity[ctf] += s->same_pid_count[oid];
        else { free(oids); free(mid_xys); return -2; }
    }
    {
        uint64_t sum = 0;
        for (uint32_t c = 0; c < C; ++c) sum += s->ctf_capacity[c];
        /* meetings longer than max_meet_time shift the reference's CTF ranges
         * off the key array: outside its domain */
        if (sum != kv) { free(oids); free(mid_xys); return -4; }
    }
    /* cuda_get_limit (:820-906) and get_ctf_bits on the host (:1950-1954) */
    memset(s->ctfs, 0, sizeof(go_ctf_meta) * C);
    uint64_t key_index = 0;
    int ok = 1;
    for (uint32_t c = 0; c < C; ++c) {
        go_ctf_meta *m = &s->ctfs[c];
        const uint64_t cap = s->ctf_capacity[c];
        uint64_t n = cap;
        if (key_index + n > cfg->kv_capacity) n = key_index < cfg->kv_capacity ? cfg->kv_capacity - key_index : 0;
        limit_counts(s, s->keys, s->boxes, key_index, n, 1, m->ctf_mbr, &m->start_time_min, &m->start_time_max);
        m->CTF_kv_capacity = (uint32_t)cap;
        m->end_time_min = s->end_time_min;
        m->end_time_max = cur_time;
        if (!ctf_bits(m, map, cfg)) ok = 0;
        key_index += cap;
    }
    if (!ok) { free(oids); free(mid_xys); return -3; }
    /* cuda_write_bitmap (:1003-1034) */
    key_index = 0;
    for (uint32_t c = 0; c < C; ++c) {
        const go_ctf_meta *m = &s->ctfs[c];
        const float *cm = m->ctf_mbr;
        for (uint64_t kid = key_index; kid < key_index + s->ctf_capacity[c] && kid < cfg->kv_capacity; ++kid) {
            const float *b = s->boxes + 4 * kid;
            volatile float ex = cm[2] - cm[0], ey = cm[3] - cm[1];
            volatile float f0 = (b[0] - cm[0]) / ex * m->x_grid, f1 = (b[1] - cm[1]) / ey * m->y_grid;
            volatile float f2 = (b[2] - cm[0]) / ex * m->x_grid, f3 = (b[3] - cm[1]) / ey * m->y_grid;
            const uint32_t l0 = sat_u32_f(f0), l1 = sat_u32_f(f1), h0 = sat_u32_f(f2), h1 = sat_u32_f(f3);
            const uint64_t base = (uint64_t)c * bit_count;
            for (uint64_t x = l0; x <= h0 && base + x < total_bits; ++x)
                for (uint64_t y = l1; y <= h1 && base + x + y * m->x_grid < total_bits; ++y)
                    set_bit(s->bitmaps, total_bits, base + x + y * m->x_grid, &outside);
        }
        key_index += s->ctf_capacity[c];
    }
    /* write_key_and_mbr (:1079-1104) */
    memset(s->ctf_keys, 0, cfg->kv_capacity * 16);
    key_index = 0;
    uint64_t bytes_index = 0;
    for (uint32_t c = 0; c < C; ++c) {
        const go_ctf_meta *m = &s->ctfs[c];
        const uint32_t kb = m->key_bit / 8;
        for (uint64_t kid = key_index; kid < key_index + s->ctf_capacity[c] && kid < cfg->kv_capacity; ++kid) {
            const u128 key = s->keys[kid];
            const u128 end = key & 0xffffffffu;
            const u128 duration = (key >> FO_END_BIT) & 0xffffffffu;
            const u128 target = (key >> (FO_DURATION_BIT + FO_END_BIT)) & ((1u << FO_OID_BIT) - 1);
            const u128 pid = key >> (FO_OID_BIT + FO_DURATION_BIT + FO_END_BIT);
            const u128 value_mbr = serialize_box(s->boxes + 4 * kid, m);
            const u128 temp = (pid << (m->id_bit + m->duration_bit + m->end_bit + m->mbr_bit)) +
                              (target << (m->duration_bit + m->end_bit + m->mbr_bit)) +
                              (duration << (m->end_bit + m->mbr_bit)) + (end << m->mbr_bit) + value_mbr;
            const uint64_t at = bytes_index + (kid - key_index) * kb;
            if (at + kb <= cfg->kv_capacity * 16) memcpy(s->ctf_keys + at, &temp, kb);
        }
        key_index += s->ctf_capacity[c];
        bytes_index += (uint64_t)s->ctf_capacity[c] * m->key_bit / 8;
    }
    memcpy(s->out_sids, s->sids, sizeof(uint16_t) * N);

    go_store_info *inf = &s->info;
    inf->kv_count = kv;
    inf->key_bytes = bytes_index;
    inf->oversize_kv_count = (uint32_t)o_n;
    inf->oversize_start_time_min = o_smin;
    inf->oversize_start_time_max = o_smax;
    inf->oversize_end_time_min = s->end_time_min;
    inf->oversize_end_time_max = cur_time;
    inf->sid_count = s->sid_count;
    inf->oversize_oid_count = s->oversize_oid_count;
    inf->end_time_min = s->end_time_min;
    inf->cur_time = cur_time;
    inf->bits_outside = outside;
    s->have_result = 1;
    if (out) *out = *inf;

    /* reset after the dump (:2112-2131) and the new window (tracing/process.cpp:271,549) */
    for (uint32_t i = 0; i < N; ++i) {
        s->o_boxs[4 * i + 0] = 100000000;
        s->o_boxs[4 * i + 1] = 100000000;
        s->o_boxs[4 * i + 2] = 0;
        s->o_boxs[4 * i + 3] = 0;
    }
    s->sid_count = 0;
    s->oversize_oid_count = 0;
    memset(s->sids, 0, sizeof(uint16_t) * N);
    memset(s->same_pid_count, 0, sizeof(uint32_t) * N);
    s->kv_count = 0;
    s->end_time_min = cur_time;
    free(oids);
    free(mid_xys);
    return 0;
}

void go_store_result(const go_store *s, uint8_t *keys, uint16_t *sids, uint32_t *ctf_capacity, go_ctf_meta *ctfs,
                     uint8_t *bitmaps, void *o_keys, float *o_boxes, uint8_t *o_bitmap) {
    const go_store_config *cfg = &s->cfg;
    const uint64_t bit_bytes = FO_BITMAP_EDGE * FO_BITMAP_EDGE / 8;
    if (keys) memcpy(keys, s->ctf_keys, s->info.key_bytes);
    if (sids) memcpy(sids, s->out_sids, sizeof(uint16_t) * cfg->num_objects);
    if (ctf_capacity) memcpy(ctf_capacity, s->ctf_capacity, sizeof(uint32_t) * cfg->CTF_count);
    if (ctfs) memcpy(ctfs, s->ctfs, sizeof(go_ctf_meta) * cfg->CTF_count);
    if (bitmaps) memcpy(bitmaps, s->bitmaps, cfg->CTF_count * bit_bytes);
    if (o_keys) memcpy(o_keys, s->o_keys, sizeof(u128) * s->info.oversize_kv_count);
    if (o_boxes) memcpy(o_boxes, s->o_boxes, sizeof(float) * 4 * s->info.oversize_kv_count);
    if (o_bitmap) memcpy(o_bitmap, s->o_bitmap, bit_bytes);
}

/* the last flush's sorted keys (CTF part, then oversize part) and boxes */
uint64_t go_store_sorted(const go_store *s, void *keys, float *boxes) {
    const uint64_t n = s->info.kv_count + s->info.oversize_kv_count;
    if (keys) memcpy(keys, s->keys, sizeof(u128) * n);
    if (boxes) memcpy(boxes, s->boxes, sizeof(float) * 4 * n);
    return n;
}

/* the CTF encoding helpers for the compaction restatement */
int go_ctf_bits(go_ctf_meta *c, const double *map4, uint32_t num_objects, uint32_t max_meet_time) {
    go_store_config cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.num_objects = num_objects;
    cfg.max_meet_time = max_meet_time;
    return ctf_bits(c, map4, &cfg);
}

uint64_t go_serialize_box(const float *box4, const go_ctf_meta *c) { return serialize_box(box4, c); }
