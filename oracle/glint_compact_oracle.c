/*
 * glint_compact_oracle.c -- CPU restatement of the reference's compaction of
 * stored contact-tracing blocks (merge_dump, tools/compaction.cpp:729-1215).
 *
 * TEST INFRASTRUCTURE: used only by tests/ and bench.py's CPU legs.
 *
 * merge_dump merges `count` consecutive blocks (CTBs) into one block of
 * split_num^2 CTFs:
 *   1. sids: 1 where any source block marks the object oversize (:742-749);
 *   2. every key of every source CTF is parsed (CTF::parse_key,
 *      new_parse_mbr_f_box, tracing/step_merge.cpp:347-398) and its end made
 *      absolute (+ the CTF's end_time_min).  A key whose object the source
 *      block marks oversize goes to an extra oversize list; any other key
 *      marks its object 2, widens the object's box (f_box::update) and joins
 *      the object's key list (:797-825);
 *   3. each object's list is sorted by target (cmp_ki, :92-97);
 *   4. STR: the objects marked 2 are sorted by the x middle of their box
 *      (compare_two_level, :139-155); split_index is the last of them, and
 *      only positions [0, split_index) are placed.  x_part = split_index /
 *      split_num + 1; each x part is sorted by y (compare_y); y_part =
 *      x_part / split_num + 1; position i goes to CTF (i / x_part) * split_num
 *      + (i % x_part) / y_part (:869-917);
 *   5. each CTF's object list has y_part entries (the last CTF
 *      split_index - x_part (split_num - 1) - y_part (split_num - 1)); the
 *      entries no position fills stay 0, so after the list's sort they
 *      repeat object 0's keys at the front of the CTF (:908-938);
 *   6. per CTF: box and start-time limits over its keys, get_ctf_bits, the
 *      bitmap, and the packed keys with end + end_time_min (:960-1063);
 *   7. the oversize buffers of the sources and the extra list are merged by
 *      repeatedly taking the smallest head key, ties to the earlier buffer;
 *      their bitmaps are OR-ed, their time limits folded with the merged
 *      buffer's zero start (:1079-1127).
 *
 * The reference sorts with std::sort, which leaves the order of equivalent
 * elements unspecified.  Two orders are offered (go_compact's std_ties):
 *   std_ties = 1: the C++ library's own std::sort with the reference's
 *     comparators (glint_compact_sort.cpp), which reproduces the reference's
 *     output bit for bit with the same library;
 *   std_ties = 0: a stable order, the device path's: objects of equal x (or
 *     y) middle keep object-id order (the x-sorted order for the y sort),
 *     keys of one object with equal targets keep the order of their source
 *     blocks and CTF positions, and so does the extra oversize list.
 * The two differ only where equivalent elements straddle a partition
 * boundary or sit side by side in one CTF.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "glint_oracle.h"

typedef unsigned __int128 u128;

#define GC_BIT_BYTES (256 * 256 / 8)   /* DEFAULT_bitmap_edge^2 / 8, util/util.h:47 */

struct go_compaction {
    uint32_t C, N;
    uint64_t kv, key_bytes, o_count, padding;
    uint32_t x_part, y_part, sid_count;
    uint16_t *sids;
    go_ctf_meta *ctfs;
    uint8_t *bitmaps;
    uint8_t *keys;
    u128 *o_keys;
    float *o_boxes;
    uint8_t o_bitmap[GC_BIT_BYTES];
    uint32_t times[8];
};

typedef struct {
    uint32_t oid, target, duration, end;
    float box[4];
    uint64_t seq;
} gc_rec;

/* CTF::parse_key (tracing/step_merge.cpp:347-357) on packed bytes */
static void parse_key(const go_ctf_meta *c, const uint8_t *p, gc_rec *r, uint64_t *value_mbr) {
    u128 k = 0;
    memcpy(&k, p, c->key_bit / 8);     /* little-endian on every host */
    *value_mbr = (uint64_t)(k & (((u128)1 << c->mbr_bit) - 1));
    k >>= c->mbr_bit;
    r->end = (uint32_t)(k & ((1ull << c->end_bit) - 1));
    k >>= c->end_bit;
    r->duration = (uint32_t)(k & ((1ull << c->duration_bit) - 1));
    k >>= c->duration_bit;
    r->target = (uint32_t)(k & ((1ull << c->id_bit) - 1));
    k >>= c->id_bit;
    /* parse_key keeps every bit above the target as the object id, but the
     * flush writes the whole 38-bit (sid, oid) field there (extract_fields,
     * cuda/cuda_util.cuh:164-169), so the packed bytes can hold sid bits above
     * the id (key_bit rounds up, N > 2^19) and merge_dump would index past
     * its object arrays; the id is read as the reference's readers read it,
     * id_bit bits (CTF::ctf_get_key_oid, tracing/step_merge.cpp:331-333) */
    r->oid = (uint32_t)(k & ((1ull << c->id_bit) - 1));
}

/* CTF::new_parse_mbr_f_box (tracing/step_merge.cpp:381-398): double
 * arithmetic, each coordinate rounded to float */
static void parse_box(const go_ctf_meta *c, uint64_t v, float *b) {
    const uint64_t mask_edge = (1ull << c->edge_bit) - 1;
    const uint64_t mask_low_y = (1ull << c->low_y_bit) - 1;
    const uint64_t mask_low_x = (1ull << c->low_x_bit) - 1;
    const uint64_t y = v & mask_edge;
    v >>= c->edge_bit;
    const uint64_t x = v & mask_edge;
    v >>= c->edge_bit;
    const uint64_t low1 = v & mask_low_y;
    v >>= c->low_y_bit;
    const uint64_t low0 = v & mask_low_x;
    const float *m = c->ctf_mbr;
    const float ex = m[2] - m[0], ey = m[3] - m[1];
    const float longer_edge = ex < ey ? ey : ex;   /* std::max */
    b[0] = (float)((double)m[0] + (double)low0 / (double)mask_low_x * (double)ex);
    b[1] = (float)((double)m[1] + (double)low1 / (double)mask_low_y * (double)ey);
    b[2] = (float)((double)b[0] + (double)x / (double)mask_edge * (double)longer_edge);
    b[3] = (float)((double)b[1] + (double)y / (double)mask_edge * (double)longer_edge);
}

/* f_box::update (geometry/geometry.h:299-312) */
static void box_update(float *acc, const float *b) {
    if (acc[0] > b[0]) acc[0] = b[0];
    if (acc[2] < b[2]) acc[2] = b[2];
    if (acc[1] > b[1]) acc[1] = b[1];
    if (acc[3] < b[3]) acc[3] = b[3];
}

static const gc_rec *g_recs;
static int cmp_rec(const void *a, const void *b) {
    const gc_rec *x = &g_recs[*(const uint64_t *)a], *y = &g_recs[*(const uint64_t *)b];
    if (x->oid != y->oid) return x->oid < y->oid ? -1 : 1;
    if (x->target != y->target) return x->target < y->target ? -1 : 1;
    return x->seq < y->seq ? -1 : (x->seq > y->seq);
}

typedef struct {
    double v;
    uint32_t oid, pos;
} gc_loc;
static int cmp_loc(const void *a, const void *b) {
    const gc_loc *x = a, *y = b;
    if (x->v < y->v) return -1;
    if (y->v < x->v) return 1;
    return x->pos < y->pos ? -1 : (x->pos > y->pos);
}
static int cmp_rec_seq(const void *a, const void *b) {
    const gc_rec *x = &g_recs[*(const uint64_t *)a], *y = &g_recs[*(const uint64_t *)b];
    if (x->oid != y->oid) return x->oid < y->oid ? -1 : 1;
    return x->seq < y->seq ? -1 : (x->seq > y->seq);
}

/* std::sort with the reference's comparators (glint_compact_sort.cpp) */
void go_cmp_std_sort_objects(const uint8_t *last, const double *ax, const double *ay, uint32_t N, uint32_t *order);
void go_cmp_std_sort_y(const double *ay, uint32_t *order, uint32_t lo, uint32_t hi);
void go_cmp_std_sort_targets(const uint32_t *target, uint64_t *idx, uint64_t n);
void go_cmp_std_sort_pairs(const uint32_t *oid, const uint32_t *target, uint64_t *idx, uint64_t n);

static int cmp_u32(const void *a, const void *b) {
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : (x > y);
}

void go_compact_free(go_compaction *h) {
    if (!h) return;
    free(h->sids);
    free(h->ctfs);
    free(h->bitmaps);
    free(h->keys);
    free(h->o_keys);
    free(h->o_boxes);
    free(h);
}

int go_compact(const go_block *blocks, uint32_t count, uint32_t N, const double *map4, uint32_t max_meet_time,
               uint32_t split_num, int std_ties, go_compaction **out) {
    *out = NULL;
    if (split_num == 0 || split_num > 255) return GO_CMP_PARTITION;
    const uint32_t s = split_num, C = s * s;
    int rc = 0;
    go_compaction *h = calloc(1, sizeof(go_compaction));
    h->C = C;
    h->N = N;
    uint8_t *cls = calloc(N, 1);
    float *obox = malloc(sizeof(float) * 4 * (size_t)N);
    uint32_t *nkeys = calloc(N, sizeof(uint32_t));
    for (uint32_t o = 0; o < N; ++o) {
        obox[4 * o + 0] = obox[4 * o + 1] = 100000.0f;
        obox[4 * o + 2] = obox[4 * o + 3] = -100000.0f;
    }
    /* 1. oversize in any source block */
    for (uint32_t i = 0; i < count; ++i)
        for (uint32_t o = 0; o < N; ++o)
            if (blocks[i].sids[o] == 1) cls[o] = 1;

    /* 2. every CTF key, block by block, CTF by CTF */
    uint64_t R = 0;
    for (uint32_t i = 0; i < count; ++i)
        for (uint32_t j = 0; j < blocks[i].CTF_count; ++j) R += blocks[i].ctfs[j].CTF_kv_capacity;
    gc_rec *recs = malloc(sizeof(gc_rec) * (R ? R : 1));
    gc_rec *extra = malloc(sizeof(gc_rec) * (R ? R : 1));
    uint64_t nr = 0, ne = 0, seq = 0;
    for (uint32_t i = 0; i < count && rc == 0; ++i) {
        const go_block *b = &blocks[i];
        const uint8_t *p = b->keys;
        for (uint32_t j = 0; j < b->CTF_count && rc == 0; ++j) {
            const go_ctf_meta *c = &b->ctfs[j];
            const uint32_t kb = c->key_bit / 8;
            for (uint32_t k = 0; k < c->CTF_kv_capacity; ++k, p += kb, ++seq) {
                gc_rec r;
                uint64_t vm;
                parse_key(c, p, &r, &vm);
                if (r.oid >= N) {
                    rc = GO_CMP_OID;
                    break;
                }
                r.end += c->end_time_min;
                parse_box(c, vm, r.box);
                r.seq = seq;
                if (b->sids[r.oid] == 1) {
                    extra[ne++] = r;
                } else {
                    cls[r.oid] = 2;
                    box_update(&obox[4 * (size_t)r.oid], r.box);
                    nkeys[r.oid]++;
                    recs[nr++] = r;
                }
            }
        }
    }
    /* 3. each object's keys by target: stable, or std::sort from source order */
    uint64_t *ord = malloc(sizeof(uint64_t) * (nr ? nr : 1));
    for (uint64_t r = 0; r < nr; ++r) ord[r] = r;
    g_recs = recs;
    if (rc == 0 && nr) qsort(ord, nr, sizeof(uint64_t), std_ties ? cmp_rec_seq : cmp_rec);
    uint64_t *first = calloc(N, sizeof(uint64_t));   /* each object's first key in ord */
    for (uint64_t r = nr; r-- > 0;) first[recs[ord[r]].oid] = r;
    if (rc == 0 && std_ties) {
        uint32_t *tg = malloc(sizeof(uint32_t) * (nr ? nr : 1));
        for (uint64_t r = 0; r < nr; ++r) tg[r] = recs[ord[r]].target;
        for (uint32_t o = 0; o < N; ++o)
            if (nkeys[o] > 1) go_cmp_std_sort_targets(tg + first[o], ord + first[o], nkeys[o]);
        free(tg);
    }

    /* 4. STR over the objects marked 2: order[0, S) */
    uint32_t S = 0;
    for (uint32_t o = 0; o < N; ++o) S += cls[o] == 2;
    uint32_t *order = malloc(sizeof(uint32_t) * (N ? N : 1));
    double *ax = calloc(N ? N : 1, sizeof(double)), *ay = calloc(N ? N : 1, sizeof(double));
    for (uint32_t o = 0; o < N; ++o)
        if (cls[o] == 2) {
            const float mx = obox[4 * o + 0] / 2 + obox[4 * o + 2] / 2;
            const float my = obox[4 * o + 1] / 2 + obox[4 * o + 3] / 2;
            ax[o] = (double)mx;
            ay[o] = (double)my;
        }
    gc_loc *loc = malloc(sizeof(gc_loc) * (S ? S : 1));
    uint32_t **lists = calloc(C, sizeof(uint32_t *));
    uint32_t *lsize = calloc(C, sizeof(uint32_t));
    if (rc == 0 && S == 0) rc = GO_CMP_NO_KEYS;
    uint32_t split = 0, x_part = 0, y_part = 0;
    if (rc == 0) {
        if (std_ties) {
            uint8_t *last = malloc(N);
            for (uint32_t o = 0; o < N; ++o) last[o] = cls[o] != 2;
            go_cmp_std_sort_objects(last, ax, ay, N, order);
            free(last);
        } else {
            uint32_t n = 0;
            for (uint32_t o = 0; o < N; ++o)
                if (cls[o] == 2) {
                    loc[n].v = ax[o];
                    loc[n].oid = o;
                    loc[n].pos = n;
                    ++n;
                }
            qsort(loc, S, sizeof(gc_loc), cmp_loc);
            for (uint32_t i = 0; i < S; ++i) order[i] = loc[i].oid;
        }
        split = S - 1;
        x_part = split / s + 1;
        y_part = x_part / s + 1;
        const int64_t last = (int64_t)split - (int64_t)x_part * (s - 1) - (int64_t)y_part * (s - 1);
        if (last < 0) rc = GO_CMP_PARTITION;
        if (rc == 0) {
            /* y sorts of the x parts; position split_index stays last */
            for (uint32_t xi = 0; xi < s; ++xi) {
                const uint32_t lo = x_part * xi, hi = xi + 1 < s ? x_part * (xi + 1) : split;
                if (hi <= lo) continue;
                if (std_ties) {
                    go_cmp_std_sort_y(ay, order, lo, hi);
                } else {
                    for (uint32_t q = lo; q < hi; ++q) {
                        loc[q - lo].v = ay[order[q]];
                        loc[q - lo].oid = order[q];
                        loc[q - lo].pos = q;
                    }
                    qsort(loc, hi - lo, sizeof(gc_loc), cmp_loc);
                    for (uint32_t q = lo; q < hi; ++q) order[q] = loc[q - lo].oid;
                }
            }
            for (uint32_t c = 0; c < C; ++c) {
                lsize[c] = c + 1 < C ? y_part : (uint32_t)last;
                lists[c] = calloc(lsize[c] ? lsize[c] : 1, sizeof(uint32_t));
            }
            for (uint32_t i = 0; i < split; ++i) {
                const uint32_t xi = i / x_part, yi = (i % x_part) / y_part;
                const uint32_t sid = xi * s + yi + 2;
                lists[sid - 2][i - xi * x_part - yi * y_part] = order[i];
            }
        }
    }
    h->sids = calloc(N, sizeof(uint16_t));
    if (rc == 0) {
        for (uint32_t o = 0; o < N; ++o) h->sids[o] = cls[o];
        for (uint32_t i = 0; i < split; ++i) {
            const uint32_t xi = i / x_part, yi = (i % x_part) / y_part;
            h->sids[order[i]] = (uint16_t)(xi * s + yi + 2);
        }
        h->x_part = x_part;
        h->y_part = y_part;
        h->sid_count = split;
    }

    /* 5.-6. the CTFs */
    uint32_t times[4] = {1u << 30, 0, 1u << 30, 0};
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t *t = blocks[i].times;
        if (t[2] < times[2]) times[2] = t[2];
        if (t[3] > times[3]) times[3] = t[3];
        if (t[0] < times[0]) times[0] = t[0];
        if (t[1] > times[1]) times[1] = t[1];
    }
    h->ctfs = calloc(C, sizeof(go_ctf_meta));
    h->bitmaps = calloc((size_t)C, GC_BIT_BYTES);
    uint64_t *cap = calloc(C, sizeof(uint64_t));
    for (uint32_t c = 0; c < C && rc == 0; ++c) {
        qsort(lists[c], lsize[c], sizeof(uint32_t), cmp_u32);
        for (uint32_t k = 0; k < lsize[c]; ++k) {
            cap[c] += nkeys[lists[c][k]];
        }
        go_ctf_meta *m = &h->ctfs[c];
        float lim[4] = {100000.0f, 100000.0f, -100000.0f, -100000.0f};
        uint32_t smin = 1u << 30, smax = 1;
        for (uint32_t k = 0; k < lsize[c]; ++k) {
            const uint32_t o = lists[c][k];
            for (uint32_t q = 0; q < nkeys[o]; ++q) {
                const gc_rec *r = &recs[ord[first[o] + q]];
                /* std::min / std::max keep the earlier value on ties */
                if (r->box[0] < lim[0]) lim[0] = r->box[0];
                if (r->box[1] < lim[1]) lim[1] = r->box[1];
                if (lim[2] < r->box[2]) lim[2] = r->box[2];
                if (lim[3] < r->box[3]) lim[3] = r->box[3];
                const uint32_t st = r->end - r->duration;
                if (st < smin) smin = st;
                if (smax < st) smax = st;
            }
        }
        memcpy(m->ctf_mbr, lim, sizeof(lim));
        m->CTF_kv_capacity = (uint32_t)cap[c];
        m->start_time_min = smin;
        m->start_time_max = smax;
        m->end_time_min = times[2];
        m->end_time_max = times[3];
        if (!go_ctf_bits(m, map4, N, max_meet_time)) rc = GO_CMP_CTF_BITS;
    }
    /* entries of the object lists that no position filled */
    if (rc == 0) {
        uint64_t placed = 0;
        for (uint32_t c = 0; c < C; ++c) placed += lsize[c];
        h->padding = placed - split;
    }
    uint64_t key_bytes = 0, kv = 0;
    for (uint32_t c = 0; c < C && rc == 0; ++c) {
        key_bytes += cap[c] * (h->ctfs[c].key_bit / 8);
        kv += cap[c];
    }
    if (rc == 0) {
        h->kv = kv;
        h->key_bytes = key_bytes;
        h->keys = malloc(key_bytes ? key_bytes : 1);
        uint8_t *p = h->keys;
        for (uint32_t c = 0; c < C; ++c) {
            const go_ctf_meta *m = &h->ctfs[c];
            const uint32_t kb = m->key_bit / 8;
            uint8_t *bits = h->bitmaps + (size_t)c * GC_BIT_BYTES;
            const float ex = m->ctf_mbr[2] - m->ctf_mbr[0], ey = m->ctf_mbr[3] - m->ctf_mbr[1];
            for (uint32_t k = 0; k < lsize[c]; ++k) {
                const uint32_t o = lists[c][k];
                for (uint32_t q = 0; q < nkeys[o]; ++q, p += kb) {
                    const gc_rec *r = &recs[ord[first[o] + q]];
                    /* the bitmap (:1018-1038) */
                    const uint32_t l0 = (uint32_t)((r->box[0] - m->ctf_mbr[0]) / ex * (float)m->x_grid);
                    const uint32_t l1 = (uint32_t)((r->box[1] - m->ctf_mbr[1]) / ey * (float)m->y_grid);
                    const uint32_t h0 = (uint32_t)((r->box[2] - m->ctf_mbr[0]) / ex * (float)m->x_grid);
                    const uint32_t h1 = (uint32_t)((r->box[3] - m->ctf_mbr[1]) / ey * (float)m->y_grid);
                    for (uint32_t mx = l0; mx <= h0 && mx < m->x_grid; ++mx)
                        for (uint32_t ny = l1; ny <= h1 && ny < m->y_grid; ++ny) {
                            const uint32_t pos = mx + ny * m->x_grid;
                            bits[pos / 8] |= (uint8_t)(1u << (pos % 8));
                        }
                    /* the key (:1049-1060): the end is made absolute once more */
                    const u128 vm = go_serialize_box(r->box, m);
                    const u128 end = (u128)r->end + m->end_time_min;
                    const u128 key = ((u128)r->oid << (m->id_bit + m->duration_bit + m->end_bit + m->mbr_bit)) +
                                     ((u128)r->target << (m->duration_bit + m->end_bit + m->mbr_bit)) +
                                     ((u128)r->duration << (m->end_bit + m->mbr_bit)) + (end << m->mbr_bit) + vm;
                    memcpy(p, &key, kb);
                }
            }
        }
    }

    /* 7. the oversize buffers */
    if (rc == 0) {
        uint64_t total = ne;
        for (uint32_t i = 0; i < count; ++i) total += blocks[i].o_count;
        h->o_count = total;
        h->o_keys = malloc(sizeof(u128) * (total ? total : 1));
        h->o_boxes = malloc(sizeof(float) * 4 * (total ? total : 1));
        /* the extra list by (oid, target), as source keys without sid bits */
        uint64_t *eo = malloc(sizeof(uint64_t) * (ne ? ne : 1));
        for (uint64_t r = 0; r < ne; ++r) eo[r] = r;
        g_recs = extra;
        if (ne && !std_ties) qsort(eo, ne, sizeof(uint64_t), cmp_rec);
        if (ne && std_ties) {
            uint32_t *eoid = malloc(sizeof(uint32_t) * ne), *etg = malloc(sizeof(uint32_t) * ne);
            for (uint64_t r = 0; r < ne; ++r) {
                eoid[r] = extra[r].oid;
                etg[r] = extra[r].target;
            }
            go_cmp_std_sort_pairs(eoid, etg, eo, ne);
            free(eoid);
            free(etg);
        }
        u128 *ek = malloc(sizeof(u128) * (ne ? ne : 1));
        float *eb = malloc(sizeof(float) * 4 * (ne ? ne : 1));
        for (uint64_t r = 0; r < ne; ++r) {
            const gc_rec *x = &extra[eo[r]];
            ek[r] = ((u128)x->oid << (26 + 32 + 32)) + ((u128)x->target << (32 + 32)) + ((u128)x->duration << 32) +
                    (u128)x->end;
            memcpy(&eb[4 * r], x->box, sizeof(float) * 4);
        }
        const uint32_t nb = count + 1;
        uint64_t *at = calloc(nb, sizeof(uint64_t));
        for (uint64_t kv2 = 0; kv2 < total; ++kv2) {
            u128 best = (u128)1 << 126;
            uint32_t taken = 0;
            for (uint32_t i = 0; i < nb; ++i) {
                const uint64_t n = i < count ? blocks[i].o_count : ne;
                if (at[i] >= n) continue;
                u128 k;
                if (i < count) memcpy(&k, blocks[i].o_keys + 16 * at[i], 16);
                else k = ek[at[i]];
                if (best > k) {
                    taken = i;
                    best = k;
                }
            }
            h->o_keys[kv2] = best;
            const float *src = taken < count ? blocks[taken].o_boxes + 4 * at[taken] : eb + 4 * at[taken];
            memcpy(&h->o_boxes[4 * kv2], src, sizeof(float) * 4);
            at[taken]++;
        }
        free(at);
        free(eo);
        free(ek);
        free(eb);
        memset(h->o_bitmap, 0, sizeof(h->o_bitmap));
        uint32_t ot[4] = {0, 0, 0, 0};
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t *t = blocks[i].o_times;
            if (t[0] < ot[0]) ot[0] = t[0];
            if (t[1] > ot[1]) ot[1] = t[1];
            if (t[2] < ot[2]) ot[2] = t[2];
            if (t[3] > ot[3]) ot[3] = t[3];
            for (uint32_t j = 0; j < GC_BIT_BYTES; ++j) h->o_bitmap[j] |= blocks[i].o_bitmap[j];
        }
        memcpy(h->times, times, sizeof(times));
        memcpy(h->times + 4, ot, sizeof(ot));
    }

    for (uint32_t c = 0; c < C; ++c) free(lists[c]);
    free(lists);
    free(lsize);
    free(cap);
    free(loc);
    free(order);
    free(ax);
    free(ay);
    free(first);
    free(ord);
    free(recs);
    free(extra);
    free(nkeys);
    free(obox);
    free(cls);
    if (rc != 0) {
        go_compact_free(h);
        return rc;
    }
    *out = h;
    return 0;
}

void go_compact_sizes(const go_compaction *h, uint64_t *sizes) {
    sizes[0] = h->C;
    sizes[1] = h->kv;
    sizes[2] = h->key_bytes;
    sizes[3] = h->o_count;
    sizes[4] = h->padding;
    sizes[5] = h->x_part;
    sizes[6] = h->y_part;
    sizes[7] = h->sid_count;
}

void go_compact_result(const go_compaction *h, uint8_t *keys, uint16_t *sids, go_ctf_meta *ctfs, uint8_t *bitmaps,
                       void *o_keys, float *o_boxes, uint8_t *o_bitmap, uint32_t *times8) {
    if (keys) memcpy(keys, h->keys, h->key_bytes);
    if (sids) memcpy(sids, h->sids, sizeof(uint16_t) * h->N);
    if (ctfs) memcpy(ctfs, h->ctfs, sizeof(go_ctf_meta) * h->C);
    if (bitmaps) memcpy(bitmaps, h->bitmaps, (size_t)h->C * GC_BIT_BYTES);
    if (o_keys) memcpy(o_keys, h->o_keys, sizeof(u128) * h->o_count);
    if (o_boxes) memcpy(o_boxes, h->o_boxes, sizeof(float) * 4 * h->o_count);
    if (o_bitmap) memcpy(o_bitmap, h->o_bitmap, GC_BIT_BYTES);
    if (times8) memcpy(times8, h->times, sizeof(uint32_t) * 8);
}
