/*
 * glint_oracle.c -- single-threaded CPU restatement of the reference's
 * per-timestep contact-tracing stages.  TEST ORACLE ONLY: imported by tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline leg, never by the
 * product path.  Build: oracle/Makefile (gcc -O2 -ffp-contract=off).
 *
 * Every function names the reference lines it follows.  Where the reference
 * runs a stage on several pthreads, this file produces the results of one
 * thread in the reference's batch order, which is the only order in which the
 * reference's results are reproducible (leaf-overflow drops and hash-slot
 * placement depend on it).
 *
 * go_set_threads(c, n) spreads the order-free parts of a step over n host
 * threads without changing any result: the descent and tree walk of each
 * object, the distance tests of each check and the scan of each bucket range
 * run in contiguous chunks, and everything whose outcome depends on order
 * (leaf inserts, meeting-table inserts and touches, report order, schema
 * update) is applied afterwards in the single-threaded order, chunk after
 * chunk.  This is what makes the oracle usable at 10M objects.
 */
#define _GNU_SOURCE
#include "glint_oracle.h"

#include <math.h>
#include <pthread.h>
#include <sys/mman.h>
#include <stdlib.h>
#include <string.h>

#define GO_PI 3.14159265                     /* util/util.h:38 */
#define GO_EMPTY_KEY (1ULL << 62)            /* util/util.h:39 (ULL_MAX) */

static const double go_dpm_lat_c = 360.0 / (40076.0 * 1000.0); /* util/util.h:57 */

double go_dpm_lat(void) { return go_dpm_lat_c; }

/* util/util.h:59-66 */
double go_dpm_lon(double latitude) {
    double absla = fabs(latitude);
    if (absla == 90) absla = 89;
    return 360.0 / (sin((90 - absla) * GO_PI / 180) * 40076.0 * 1000.0);
}

/* util/util.h:68-70 */
uint64_t go_cantor(uint32_t pid1, uint32_t pid2) {
    return (uint64_t)(pid1 + pid2) * (pid1 + pid2 + 1) / 2 + pid2;
}

/* exact integer inverse of go_cantor (the reference's InverseCantorPairing1,
 * util/util.h:72-78, uses a floating sqrt; this one corrects it to the exact
 * triangular root) */
void go_cantor_inverse(uint64_t z, uint32_t *a, uint32_t *b) {
    uint64_t w = (uint64_t)floor((sqrt(8.0 * (double)z + 1) - 1) / 2);
    while (w > 0 && w * (w + 1) / 2 > z) w--;
    while ((w + 1) * (w + 2) / 2 <= z) w++;
    uint64_t t = w * (w + 1) / 2;
    uint32_t y = (uint32_t)(z - t);
    *b = y;
    *a = (uint32_t)(w - y);
}

/* ---- correctly rounded sin via double-double Taylor series ------------- */
typedef struct { double hi, lo; } dd;

static dd dd_two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    dd r = {s, e};
    return r;
}
static dd dd_quick(double a, double b) {
    double s = a + b;
    dd r = {s, b - (s - a)};
    return r;
}
static dd dd_add(dd a, dd b) {
    dd s = dd_two_sum(a.hi, b.hi);
    dd t = dd_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = dd_quick(s.hi, s.lo);
    s.lo += t.lo;
    return dd_quick(s.hi, s.lo);
}
static dd dd_mul(dd a, dd b) {
    double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e += a.hi * b.lo + a.lo * b.hi;
    return dd_quick(p, e);
}
static dd dd_div_d(dd a, double d) {
    double q1 = a.hi / d;
    double p = q1 * d;
    double pe = fma(q1, d, -p);
    double r = ((a.hi - p) - pe) + a.lo;
    double q2 = r / d;
    return dd_quick(q1, q2);
}

/* sin(x) for 0 <= x <= pi/2 (the only range the reference's formula uses):
 * Horner evaluation of the Taylor series to x^41/41! in double-double */
double go_sin_cr(double x) {
    dd xd = {x, 0.0};
    dd x2 = dd_mul(xd, xd);
    /* coefficients (-1)^k/(2k+1)! for k = 0..20 */
    dd coef[21];
    dd f = {1.0, 0.0};
    coef[0] = f;
    for (int k = 1; k <= 20; ++k) {
        f = dd_div_d(f, (double)(2 * k));
        f = dd_div_d(f, (double)(2 * k + 1));
        dd c = f;
        if (k & 1) { c.hi = -c.hi; c.lo = -c.lo; }
        coef[k] = c;
    }
    dd acc = coef[20];
    for (int k = 19; k >= 0; --k) acc = dd_add(dd_mul(acc, x2), coef[k]);
    acc = dd_mul(acc, xd);
    return acc.hi + acc.lo;
}

/* ---- context ------------------------------------------------------------ */
typedef struct go_check {
    uint32_t pid;
    uint32_t gid;
    uint32_t inside;
} go_check;

/* one meeting bucket: meeting_unit's key, start, end and the GPU rule's f32
 * box (tracing/workbench.h:62-83), kept together so that a probe touches
 * one cache line */
typedef struct go_rec {
    uint64_t key;
    uint32_t start, end;
    float mbr[4];
} go_rec;

#define GO_MAX_THREADS_SHARDS 64

/* growable per-thread buffers of one chunk's results */
typedef struct go_tbuf {
    go_check *checks;              /* cross checks of the chunk's objects, in order */
    size_t n_checks, cap_checks;
    uint64_t *contacts;            /* (checking pid << 32) | member, in test order */
    size_t n_contacts, cap_contacts;
    go_meeting *reports;           /* meetings of the chunk's buckets, in bucket order */
    size_t n_reports, cap_reports;
    uint64_t candidates, taken;
    uint32_t active;
    /* the chunk's contacts split by a lookup in the table as it stood before
     * the step: pairs found there (with their slot), by the slot range that
     * owns the slot, and pairs not found (in test order) */
    uint64_t *touch[2 * GO_MAX_THREADS_SHARDS];
    size_t n_touch[GO_MAX_THREADS_SHARDS], cap_touch[GO_MAX_THREADS_SHARDS];
    uint64_t *fresh[GO_MAX_THREADS_SHARDS];   /* (order, pair) of pairs not found, by home slot range */
    size_t n_fresh[GO_MAX_THREADS_SHARDS], cap_fresh[GO_MAX_THREADS_SHARDS];
} go_tbuf;

/* one undo record of a slot range's inserts and touches */
typedef struct go_undo {
    uint64_t slot;
    go_rec old;
} go_undo;

/* one slot range of the table while the pairs not found before the step are
 * inserted: probes that reach the range's end leave (out) and enter the
 * next range at its first slot (in) */
typedef struct go_shard {
    uint64_t *in, *used, *out;        /* (order, pair), ascending order */
    size_t n_in, cap_in, n_used, cap_used, n_out, cap_out;
    go_undo *undo;
    size_t n_undo, cap_undo;
} go_shard;

#define GO_MAX_THREADS GO_MAX_THREADS_SHARDS

struct go_ctx {
    go_config cfg;
    double mbr[4];
    double x_buffer, y_buffer;
    const double *pts;                 /* current step's points (borrowed) */
    uint32_t cur_time;

    uint32_t grid_capacity;            /* leaf buffer size */
    uint32_t grids_stack_capacity;
    uint32_t schema_stack_capacity;
    uint32_t grids_stack_index;
    uint32_t schema_stack_index;
    uint32_t *grids;                   /* [grids_stack_capacity * grid_capacity] */
    double *grid_xy;                   /* members' coordinates, grid-major (this step) */
    uint32_t *grid_counter;
    uint32_t *grids_stack;
    uint32_t *schema_stack;
    go_schema *schema;

    go_check *checks;
    size_t n_checks, cap_checks;

    go_rec *tab;                       /* [B] */
    uint32_t *obj_gid;                 /* leaf grid of each object this step */
    uint32_t threads;
    go_tbuf tb[GO_MAX_THREADS];
    go_shard sh[GO_MAX_THREADS_SHARDS];
    uint32_t shard_rounds;             /* re-runs of slot ranges in the last step */
    uint32_t *chunk_counts;            /* [threads * grids_stack_capacity] leaf insert offsets */

    go_meeting *meetings;              /* identified in the last step */
    uint32_t n_meetings, cap_meetings;
    uint64_t num_taken;
    uint32_t num_active;
    uint64_t contacts, candidates;
    uint32_t n_splits, n_merges;
};

typedef void (*go_task_fn)(go_ctx *c, uint32_t tid, uint32_t nt);
static void go_parallel(go_ctx *c, go_task_fn fn);
static void chunk_of(size_t n, uint32_t tid, uint32_t nt, size_t *lo, size_t *hi);

static double pt_x(const go_ctx *c, uint32_t pid) { return c->pts[2 * (size_t)pid]; }
static double pt_y(const go_ctx *c, uint32_t pid) { return c->pts[2 * (size_t)pid + 1]; }

/* box::distance(p, true), geometry/geometry.h:174-185 */
static double box_distance(const go_schema *s, double px, double py) {
    if (px >= s->low[0] && px <= s->high[0] && py >= s->low[1] && py <= s->high[1]) return 0;
    double ax = fabs(px - (s->low[0] + s->high[0]) / 2) - (s->high[0] - s->low[0]) / 2;
    double ay = fabs(py - (s->low[1] + s->high[1]) / 2) - (s->high[1] - s->low[1]) / 2;
    double dx = ax < 0.0 ? 0.0 : ax;  /* std::max(a, 0.0) */
    double dy = ay < 0.0 ? 0.0 : ay;
    dy = dy / go_dpm_lat_c;
    dx = dx / go_dpm_lon(py);
    return sqrt(dx * dx + dy * dy);
}

/* box::width(true), geometry/geometry.h:166-172 */
static double box_width_m(const double *low, const double *high) {
    return (high[0] - low[0]) / go_dpm_lon(low[1]);
}

/* ---- initial schema: QTNode insert/split/create_schema ------------------ */
typedef struct qt_node {
    double low[2], high[2], mid_x, mid_y;
    int16_t level;
    int isleaf;
    uint32_t node_id;
    struct qt_node *child[4];
} qt_node;

static qt_node *qt_new(double lx, double ly, double hx, double hy, int16_t level) {
    qt_node *n = (qt_node *)calloc(1, sizeof(qt_node));
    n->low[0] = lx; n->low[1] = ly; n->high[0] = hx; n->high[1] = hy;
    n->mid_x = (n->high[0] + n->low[0]) / 2;     /* index/QTree.h:103-104 */
    n->mid_y = (n->high[1] + n->low[1]) / 2;
    n->level = level;
    n->isleaf = 1;
    return n;
}

/* A node becomes a branch iff at least grid_capacity objects route to it and
 * width(true)/2 > reach (index/QTree.h:157-185); the reference's concurrent
 * inserts reach the same final tree because a node's routed count does not
 * depend on insertion order. */
static void qt_build(go_ctx *c, qt_node *n, uint32_t *ids, size_t cnt, uint32_t *scratch) {
    if (!(cnt >= c->cfg.grid_capacity && box_width_m(n->low, n->high) / 2 > c->cfg.reach_distance)) return;
    n->isleaf = 0;
    n->child[0] = qt_new(n->low[0], n->low[1], n->mid_x, n->mid_y, n->level + 1);
    n->child[1] = qt_new(n->mid_x, n->low[1], n->high[0], n->mid_y, n->level + 1);
    n->child[2] = qt_new(n->low[0], n->mid_y, n->mid_x, n->high[1], n->level + 1);
    n->child[3] = qt_new(n->mid_x, n->mid_y, n->high[0], n->high[1], n->level + 1);
    size_t counts[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < cnt; ++i) {
        double x = pt_x(c, ids[i]), y = pt_y(c, ids[i]);
        counts[(y > n->mid_y) * 2 + (x > n->mid_x)]++;
    }
    size_t off[4];
    off[0] = 0;
    for (int k = 1; k < 4; ++k) off[k] = off[k - 1] + counts[k - 1];
    size_t pos[4] = {off[0], off[1], off[2], off[3]};
    for (size_t i = 0; i < cnt; ++i) {
        double x = pt_x(c, ids[i]), y = pt_y(c, ids[i]);
        scratch[pos[(y > n->mid_y) * 2 + (x > n->mid_x)]++] = ids[i];
    }
    memcpy(ids, scratch, cnt * sizeof(uint32_t));
    for (int k = 0; k < 4; ++k) qt_build(c, n->child[k], ids + off[k], counts[k], scratch + off[k]);
}

static void qt_set_id(qt_node *n, uint32_t *id) {       /* index/QTree.h:88-96 */
    if (n->isleaf) n->node_id = (*id)++;
    else for (int k = 0; k < 4; ++k) qt_set_id(n->child[k], id);
}

static void qt_counts(qt_node *n, uint32_t *nodes, uint32_t *leaves) {
    (*nodes)++;
    if (n->isleaf) (*leaves)++;
    else for (int k = 0; k < 4; ++k) qt_counts(n->child[k], nodes, leaves);
}

static void qt_create_schema(qt_node *n, go_schema *schema, uint32_t *offset) { /* index/QTree.h:286-311 */
    uint32_t cur = (*offset)++;
    go_schema *s = &schema[cur];
    memset(s, 0, sizeof(*s));
    s->mid_x = n->mid_x;
    s->mid_y = n->mid_y;
    s->level = n->level;
    s->grid_id = n->isleaf ? n->node_id : 0;
    s->type = n->isleaf ? GO_LEAF : GO_BRANCH;
    s->low[0] = n->low[0]; s->low[1] = n->low[1];
    s->high[0] = n->high[0]; s->high[1] = n->high[1];
    if (!n->isleaf) {
        for (int k = 0; k < 4; ++k) {
            schema[cur].children[k] = *offset;
            qt_create_schema(n->child[k], schema, offset);
        }
    }
}

static void qt_free(qt_node *n) {
    if (!n->isleaf) for (int k = 0; k < 4; ++k) qt_free(n->child[k]);
    free(n);
}

/* the bucket table, on 2-MB boundaries and advised into huge pages, so
 * that random probes of a table of tens of GB do not also miss the TLB */
static go_rec *alloc_table(size_t B) {
    size_t bytes = B * sizeof(go_rec);
    size_t huge = (size_t)2 << 20;
    bytes = (bytes + huge - 1) / huge * huge;
    go_rec *t = (go_rec *)aligned_alloc(huge, bytes);
    if (t) madvise(t, bytes, MADV_HUGEPAGE);
    return t;
}

static void table_clear_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->cfg.num_meeting_buckets, tid, nt, &lo, &hi);
    memset(c->tab + lo, 0, (hi - lo) * sizeof(go_rec));
    for (size_t i = lo; i < hi; ++i) c->tab[i].key = GO_EMPTY_KEY;
}

go_ctx *go_create(const go_config *cfg, const double *mbr4, const double *points_xy) {
    return go_create_threads(cfg, mbr4, points_xy, 1);
}

go_ctx *go_create_threads(const go_config *cfg, const double *mbr4, const double *points_xy, uint32_t threads) {
    go_ctx *c = (go_ctx *)calloc(1, sizeof(go_ctx));
    c->cfg = *cfg;
    go_set_threads(c, threads);
    memcpy(c->mbr, mbr4, sizeof(c->mbr));
    /* tracing/filter.cpp:30-31 */
    c->x_buffer = cfg->reach_distance * go_dpm_lon(mbr4[1]);
    c->y_buffer = cfg->reach_distance * go_dpm_lat_c;
    /* tracing/workbench.cpp:36-47 */
    c->grid_capacity = (uint32_t)(cfg->grid_amplify * cfg->grid_capacity);
    uint32_t per = cfg->num_objects / cfg->grid_capacity;
    c->grids_stack_capacity = 4 * (per > 100000u ? per : 100000u);
    c->schema_stack_capacity = (uint32_t)(1.6 * c->grids_stack_capacity);
    /* tracing/workbench.cpp:87-129 */
    c->grids = (uint32_t *)calloc((size_t)c->grids_stack_capacity * c->grid_capacity, sizeof(uint32_t));
    c->grid_counter = (uint32_t *)calloc(c->grids_stack_capacity, sizeof(uint32_t));
    c->grid_xy = (double *)malloc(sizeof(double) * 2 * (size_t)c->grids_stack_capacity * c->grid_capacity);
    c->grids_stack = (uint32_t *)malloc(sizeof(uint32_t) * c->grids_stack_capacity);
    for (uint32_t i = 0; i < c->grids_stack_capacity; ++i) c->grids_stack[i] = i;
    c->schema = (go_schema *)calloc(c->schema_stack_capacity, sizeof(go_schema));
    c->schema_stack = (uint32_t *)malloc(sizeof(uint32_t) * c->schema_stack_capacity);
    for (uint32_t i = 0; i < c->schema_stack_capacity; ++i) {
        c->schema_stack[i] = i;
        c->schema[i].type = GO_INVALID;
    }
    size_t B = cfg->num_meeting_buckets;
    c->tab = alloc_table(B ? B : 1);
    go_parallel(c, table_clear_chunk);
    c->obj_gid = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(cfg->num_objects ? cfg->num_objects : 1));
    c->cap_meetings = cfg->num_objects * 10;   /* h_meetings_ps, workbench.cpp:167-170 */
    c->meetings = (go_meeting *)malloc(sizeof(go_meeting) * (size_t)(c->cap_meetings ? c->cap_meetings : 1));
    c->cap_checks = (size_t)cfg->num_objects * 2 + 16;
    c->checks = (go_check *)malloc(sizeof(go_check) * c->cap_checks);

    /* tracing/filter.cpp:27-93: build the QTree from the first step's points */
    c->pts = points_xy;
    uint32_t n = cfg->num_objects;
    uint32_t *ids = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t *scratch = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    qt_node *root = qt_new(mbr4[0], mbr4[1], mbr4[2], mbr4[3], 0);
    qt_build(c, root, ids, n, scratch);
    uint32_t id = 0;
    qt_set_id(root, &id);
    uint32_t nodes = 0, leaves = 0;
    qt_counts(root, &nodes, &leaves);
    c->schema_stack_index = nodes;
    c->grids_stack_index = leaves;
    uint32_t off = 0;
    qt_create_schema(root, c->schema, &off);
    qt_free(root);
    free(ids);
    free(scratch);
    c->pts = NULL;
    return c;
}

void go_destroy(go_ctx *c) {
    if (!c) return;
    free(c->grids); free(c->grid_xy); free(c->grid_counter); free(c->chunk_counts); free(c->grids_stack); free(c->schema); free(c->schema_stack);
    free(c->checks); free(c->tab); free(c->obj_gid); free(c->meetings);
    for (uint32_t t = 0; t < GO_MAX_THREADS; ++t) {
        free(c->tb[t].checks); free(c->tb[t].contacts); free(c->tb[t].reports);
        for (uint32_t j = 0; j < GO_MAX_THREADS_SHARDS; ++j) { free(c->tb[t].touch[j]); free(c->tb[t].fresh[j]); }
    }
    for (uint32_t j = 0; j < GO_MAX_THREADS_SHARDS; ++j) {
        free(c->sh[j].in); free(c->sh[j].used); free(c->sh[j].out); free(c->sh[j].undo);
    }
    free(c);
}

/* ---- host threads: contiguous chunks, joined before anything order-dependent */
typedef struct go_task { go_ctx *c; go_task_fn fn; uint32_t tid, nt; } go_task;

static void *go_task_main(void *p) {
    go_task *t = (go_task *)p;
    t->fn(t->c, t->tid, t->nt);
    return NULL;
}

static void go_parallel(go_ctx *c, go_task_fn fn) {
    uint32_t nt = c->threads;
    if (nt <= 1) { fn(c, 0, 1); return; }
    pthread_t th[GO_MAX_THREADS];
    go_task tk[GO_MAX_THREADS];
    uint32_t started = 0;
    for (uint32_t i = 1; i < nt; ++i) {
        tk[i].c = c; tk[i].fn = fn; tk[i].tid = i; tk[i].nt = nt;
        if (pthread_create(&th[i], NULL, go_task_main, &tk[i]) != 0) break;
        started = i;
    }
    fn(c, 0, nt);
    for (uint32_t i = 1; i <= started; ++i) pthread_join(th[i], NULL);
    /* chunks whose thread could not start run here, in order */
    for (uint32_t i = started + 1; i < nt; ++i) fn(c, i, nt);
}

static void chunk_of(size_t n, uint32_t tid, uint32_t nt, size_t *lo, size_t *hi) {
    size_t per = (n + nt - 1) / nt;
    *lo = per * tid < n ? per * tid : n;
    *hi = *lo + per < n ? *lo + per : n;
}

void go_set_threads(go_ctx *c, uint32_t n) {
    c->threads = n < 1 ? 1 : (n > GO_MAX_THREADS ? GO_MAX_THREADS : n);
    free(c->chunk_counts);
    c->chunk_counts = NULL;
}

static void *grow(void *p, size_t *cap, size_t need, size_t elem) {
    if (need <= *cap) return p;
    size_t nc = *cap ? *cap : 1024;
    while (nc < need) nc *= 2;
    *cap = nc;
    return realloc(p, nc * elem);
}

static void push_check(go_tbuf *b, uint32_t pid, uint32_t gid, uint32_t inside) {
    b->checks = (go_check *)grow(b->checks, &b->cap_checks, b->n_checks + 1, sizeof(go_check));
    go_check *k = &b->checks[b->n_checks++];
    k->pid = pid; k->gid = gid; k->inside = inside;
}

/* lookup_rec, tracing/filter.cpp:130-152 (query_all == false) */
static void lookup_rec(const go_ctx *c, go_tbuf *b, double px, double py, uint32_t pid, uint32_t curnode) {
    for (int i = 0; i < 4; ++i) {
        uint32_t child = c->schema[curnode].children[i];
        const go_schema *s = &c->schema[child];
        double dist = box_distance(s, px, py);
        if (dist <= c->cfg.reach_distance) {
            if (s->type == GO_LEAF) {
                if (py < s->low[1] || (py < s->high[1] && px < s->low[0]))
                    push_check(b, pid, s->grid_id, 0);
            } else {
                lookup_rec(c, b, px, py, pid, child);
            }
        }
    }
}

/* filter_unit's phased descent and tree walk (tracing/filter.cpp:228-261)
 * over one chunk of objects: each object's leaf grid, and its cross checks
 * in object order.  Only the schema is read. */
static void filter_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->cfg.num_objects, tid, nt, &lo, &hi);
    go_tbuf *b = &c->tb[tid];
    b->n_checks = 0;
    for (size_t p = lo; p < hi; ++p) {
        uint32_t pid = (uint32_t)p;
        double px = pt_x(c, pid), py = pt_y(c, pid);
        uint32_t curnode = 0, last_valid = 0;
        for (;;) {
            const go_schema *cs = &c->schema[curnode];
            int child = (py > cs->mid_y) * 2 + (px > cs->mid_x);
            curnode = cs->children[child];
            const go_schema *s = &c->schema[curnode];
            if (px + c->x_buffer < s->high[0] && py + c->y_buffer < s->high[1]) last_valid = curnode;
            if (s->type == GO_LEAF) break;
        }
        c->obj_gid[pid] = c->schema[curnode].grid_id;
        if (last_valid != curnode) lookup_rec(c, b, px, py, pid, last_valid);
    }
}

static void leaf_count_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->cfg.num_objects, tid, nt, &lo, &hi);
    uint32_t *cnt = c->chunk_counts + (size_t)tid * c->grids_stack_capacity;
    memset(cnt, 0, sizeof(uint32_t) * c->grids_stack_capacity);
    for (size_t p = lo; p < hi; ++p) cnt[c->obj_gid[p]]++;
}

static void leaf_offset_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->grids_stack_capacity, tid, nt, &lo, &hi);
    for (size_t g = lo; g < hi; ++g) {
        uint32_t run = 0;
        for (uint32_t t = 0; t < nt; ++t) {
            uint32_t *cnt = c->chunk_counts + (size_t)t * c->grids_stack_capacity + g;
            uint32_t v = *cnt;
            *cnt = run;
            run += v;
        }
        c->grid_counter[g] = run;
    }
}

static void leaf_place_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->cfg.num_objects, tid, nt, &lo, &hi);
    uint32_t *pos = c->chunk_counts + (size_t)tid * c->grids_stack_capacity;
    for (size_t p = lo; p < hi; ++p) {
        uint32_t gid = c->obj_gid[p];
        uint32_t at = pos[gid]++;
        if (at < c->grid_capacity) c->grids[(size_t)c->grid_capacity * gid + at] = (uint32_t)p;
    }
}

/* workbench::filter + filter_unit (phased), tracing/filter.cpp:209-313.
 * The leaf inserts (workbench::insert, :95-111) run in object order, as one
 * thread makes them; the inside check of object pid is checks[pid]; the
 * cross checks follow in object order. */
static void stage_filter(go_ctx *c) {
    uint32_t n = c->cfg.num_objects;
    go_parallel(c, filter_chunk);
    size_t total = n;
    for (uint32_t t = 0; t < c->threads; ++t) total += c->tb[t].n_checks;
    if (c->cap_checks < total) {
        c->cap_checks = total + total / 4 + 16;
        c->checks = (go_check *)realloc(c->checks, sizeof(go_check) * c->cap_checks);
    }
    if (c->threads == 1) {
        for (uint32_t pid = 0; pid < n; ++pid) {
            uint32_t gid = c->obj_gid[pid];
            uint32_t cur_size = c->grid_counter[gid]++;
            if (cur_size < c->grid_capacity) c->grids[(size_t)c->grid_capacity * gid + cur_size] = pid;
        }
    } else {
        /* the same inserts as a stable counting sort: each chunk's count per
         * grid, the chunks' offsets per grid, then each chunk places its
         * objects after those of the chunks before it */
        if (!c->chunk_counts)
            c->chunk_counts = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)c->threads * c->grids_stack_capacity);
        go_parallel(c, leaf_count_chunk);
        go_parallel(c, leaf_offset_chunk);
        go_parallel(c, leaf_place_chunk);
    }
    for (uint32_t pid = 0; pid < n; ++pid) {
        c->checks[pid].pid = pid;
        c->checks[pid].gid = c->obj_gid[pid];
        c->checks[pid].inside = 1;
    }
    size_t k = n;
    for (uint32_t t = 0; t < c->threads; ++t) {
        memcpy(c->checks + k, c->tb[t].checks, sizeof(go_check) * c->tb[t].n_checks);
        k += c->tb[t].n_checks;
    }
    c->n_checks = k;                              /* grid_check_counter */
}

static void mbr_update_by_point(float *m, double x, double y) { /* cuda/geometry.cu:82-96 */
    if (m[0] > x) m[0] = (float)x;
    if (m[2] < x) m[2] = (float)x;
    if (m[1] > y) m[1] = (float)y;
    if (m[3] < y) m[3] = (float)y;
}

/* coordinates of every grid's stored members, in member order, so that the
 * distance tests read them contiguously */
static void gather_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->grids_stack_capacity, tid, nt, &lo, &hi);
    for (size_t g = lo; g < hi; ++g) {
        uint32_t size = c->grid_counter[g] < c->grid_capacity ? c->grid_counter[g] : c->grid_capacity;
        const uint32_t *members = c->grids + (size_t)c->grid_capacity * g;
        double *xy = c->grid_xy + 2 * (size_t)c->grid_capacity * g;
        for (uint32_t i = 0; i < size; ++i) {
            xy[2 * i] = pt_x(c, members[i]);
            xy[2 * i + 1] = pt_y(c, members[i]);
        }
    }
}

/* the distance tests of reachability_unit (tracing/refinement.cpp:19-31)
 * over one chunk of checks: the pairs in contact, in test order.  The test
 * is Point::distance(p1, p2, true) (geometry/geometry.h:40-48) with p1 the
 * checking object; its degree_per_meter_longitude(p1.y) depends only on
 * the check, so it is taken once per check (the same value). */
static void refine_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->n_checks, tid, nt, &lo, &hi);
    go_tbuf *b = &c->tb[tid];
    b->n_contacts = 0;
    b->candidates = 0;
    const double r = c->cfg.reach_distance;
    for (size_t k = lo; k < hi; ++k) {
        uint32_t pid = c->checks[k].pid, gid = c->checks[k].gid;
        uint32_t size = c->grid_counter[gid] < c->grid_capacity ? c->grid_counter[gid] : c->grid_capacity;
        const uint32_t *members = c->grids + (size_t)c->grid_capacity * gid;
        const double *xy = c->grid_xy + 2 * (size_t)c->grid_capacity * gid;
        const int inside = c->checks[k].inside;
        double x1 = pt_x(c, pid), y1 = pt_y(c, pid);
        double lon = go_dpm_lon(y1);
        for (uint32_t i = 0; i < size; ++i) {
            uint32_t m = members[i];
            if (!(pid < m || !inside)) continue;
            b->candidates++;
            double dx = x1 - xy[2 * i];
            double dy = y1 - xy[2 * i + 1];
            dy = dy / go_dpm_lat_c;
            dx = dx / lon;
            if (sqrt(dx * dx + dy * dy) <= r) {
                b->contacts = (uint64_t *)grow(b->contacts, &b->cap_contacts, b->n_contacts + 1, sizeof(uint64_t));
                b->contacts[b->n_contacts++] = ((uint64_t)pid << 32) | m;
            }
        }
    }
}

static uint64_t contact_slot(uint64_t pm, uint64_t B) {
    uint32_t pid = (uint32_t)(pm >> 32), m = (uint32_t)pm;
    return go_cantor(pid < m ? pid : m, pid < m ? m : pid) % B;
}

static size_t shard_size(const go_ctx *c) {
    return (c->cfg.num_meeting_buckets + c->threads - 1) / c->threads;
}

/* one contact applied to the table as tracing/refinement.cpp:34-55 does:
 * probe from the home slot, touch the pair's bucket (end = t and the GPU
 * rule's box update with p1 = the checking object first,
 * cuda/geometry.cu:469-491) or start a meeting in the first empty one */
static void apply_contact(go_ctx *c, uint64_t pm, uint64_t slot) {
    const uint64_t B = c->cfg.num_meeting_buckets;
    uint32_t pid = (uint32_t)(pm >> 32), m = (uint32_t)pm;
    double x1 = pt_x(c, pid), y1 = pt_y(c, pid);
    double x2 = pt_x(c, m), y2 = pt_y(c, m);
    uint64_t key = go_cantor(pid < m ? pid : m, pid < m ? m : pid);
    for (;;) {
        go_rec *r = &c->tab[slot];
        if (r->key == key) {
            r->end = c->cur_time;
            mbr_update_by_point(r->mbr, x1, y1);
            mbr_update_by_point(r->mbr, x2, y2);
            return;
        } else if (r->key == GO_EMPTY_KEY) {
            r->key = key;
            r->start = c->cur_time;
            r->end = c->cur_time;
            r->mbr[0] = 100000.0f; r->mbr[1] = 100000.0f; r->mbr[2] = -100000.0f; r->mbr[3] = -100000.0f;
            mbr_update_by_point(r->mbr, x1, y1);
            mbr_update_by_point(r->mbr, x2, y2);
            return;
        }
        slot = (slot + 1) % B;
    }
}

enum { AHEAD = 24 };

static void prefetch_points(const go_ctx *c, uint64_t pm) {
    __builtin_prefetch(&c->pts[2 * (size_t)(pm >> 32)], 0);
    __builtin_prefetch(&c->pts[2 * (size_t)(uint32_t)pm], 0);
}

/* Lookup of one chunk's contacts in the table as it stands before any of
 * this step's inserts (read only).  A pair found there is found by every
 * one of its contacts in the sequential order too: the slots its probe
 * passes stay filled during the step and inserts fill empty slots only.
 * Its touches change that one record and nothing any probe reads, so they
 * can be applied per slot range, in order within each record.  Pairs not
 * found are applied afterwards in the sequential order. */
static void classify_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    (void)nt;
    const uint64_t B = c->cfg.num_meeting_buckets;
    const size_t per = shard_size(c);
    go_tbuf *b = &c->tb[tid];
    for (uint32_t j = 0; j < c->threads; ++j) b->n_touch[j] = b->n_fresh[j] = 0;
    uint64_t ord0 = 0;
    for (uint32_t t = 0; t < tid; ++t) ord0 += c->tb[t].n_contacts;
    for (size_t i = 0; i < b->n_contacts; ++i) {
        if (i + AHEAD < b->n_contacts) __builtin_prefetch(&c->tab[contact_slot(b->contacts[i + AHEAD], B)], 0);
        uint64_t pm = b->contacts[i];
        uint32_t pid = (uint32_t)(pm >> 32), m = (uint32_t)pm;
        uint64_t key = go_cantor(pid < m ? pid : m, pid < m ? m : pid);
        uint64_t slot = key % B;
        int found = 0;
        for (;;) {
            uint64_t k = c->tab[slot].key;
            if (k == key) { found = 1; break; }
            if (k == GO_EMPTY_KEY) break;
            slot = (slot + 1) % B;
        }
        if (found) {
            uint32_t j = (uint32_t)(slot / per);
            b->touch[j] = (uint64_t *)grow(b->touch[j], &b->cap_touch[j], 2 * (b->n_touch[j] + 1), sizeof(uint64_t));
            b->touch[j][2 * b->n_touch[j]] = pm;
            b->touch[j][2 * b->n_touch[j] + 1] = slot;
            b->n_touch[j]++;
        } else {
            uint32_t j = (uint32_t)((key % B) / per);
            b->fresh[j] = (uint64_t *)grow(b->fresh[j], &b->cap_fresh[j], 2 * (b->n_fresh[j] + 1), sizeof(uint64_t));
            b->fresh[j][2 * b->n_fresh[j]] = ord0 + i;
            b->fresh[j][2 * b->n_fresh[j] + 1] = pm;
            b->n_fresh[j]++;
        }
    }
}

/* the touches of pairs found before the step whose slot lies in slot range
 * `tid`, chunk after chunk (= test order) */
static void touch_shard(go_ctx *c, uint32_t tid, uint32_t nt) {
    (void)nt;
    for (uint32_t t = 0; t < c->threads; ++t) {
        const go_tbuf *b = &c->tb[t];
        const uint64_t *v = b->touch[tid];
        for (size_t i = 0; i < b->n_touch[tid]; ++i) {
            if (i + AHEAD < b->n_touch[tid]) {
                __builtin_prefetch(&c->tab[v[2 * (i + AHEAD) + 1]], 1);
                prefetch_points(c, v[2 * (i + AHEAD)]);
            }
            apply_contact(c, v[2 * i], v[2 * i + 1]);
        }
    }
}

/* The pairs not found before the step whose home slot lies in slot range
 * j, plus the probes entering the range from the one before (sh->in), in
 * test order: each probe walks the range as tracing/refinement.cpp:34-55
 * does, touching its pair's bucket or filling the first empty one; a probe
 * that reaches the range's end is handed on (sh->out).  Probes change only
 * slots of their own range and the range's state depends only on the probes
 * that walk it, so a range given the right entering probes ends as the
 * sequential order leaves it.  Every change is recorded so that the range
 * can be run again when its entering probes change. */
static void shard_run(go_ctx *c, uint32_t j) {
    const uint64_t B = c->cfg.num_meeting_buckets;
    const size_t per = shard_size(c);
    const uint64_t lo = (uint64_t)j * per, hi = lo + per < B ? lo + per : B;
    go_shard *sh = &c->sh[j];
    while (sh->n_undo) {
        sh->n_undo--;
        c->tab[sh->undo[sh->n_undo].slot] = sh->undo[sh->n_undo].old;
    }
    sh->n_out = 0;
    uint32_t t = 0;
    size_t i = 0, k = 0;
    for (;;) {
        while (t < c->threads && i >= c->tb[t].n_fresh[j]) { ++t; i = 0; }
        int own = t < c->threads;
        if (!own && k >= sh->n_used) break;
        uint64_t ord, pm, slot;
        if (own && (k >= sh->n_used || c->tb[t].fresh[j][2 * i] < sh->used[2 * k])) {
            ord = c->tb[t].fresh[j][2 * i];
            pm = c->tb[t].fresh[j][2 * i + 1];
            slot = contact_slot(pm, B);
            if (i + AHEAD < c->tb[t].n_fresh[j]) {
                __builtin_prefetch(&c->tab[contact_slot(c->tb[t].fresh[j][2 * (i + AHEAD) + 1], B)], 1);
                prefetch_points(c, c->tb[t].fresh[j][2 * (i + AHEAD) + 1]);
            }
            ++i;
        } else {
            ord = sh->used[2 * k];
            pm = sh->used[2 * k + 1];
            slot = lo;
            ++k;
        }
        uint32_t pid = (uint32_t)(pm >> 32), m = (uint32_t)pm;
        uint64_t key = go_cantor(pid < m ? pid : m, pid < m ? m : pid);
        while (slot < hi && c->tab[slot].key != key && c->tab[slot].key != GO_EMPTY_KEY) ++slot;
        if (slot == hi) {
            sh->out = (uint64_t *)grow(sh->out, &sh->cap_out, 2 * (sh->n_out + 1), sizeof(uint64_t));
            sh->out[2 * sh->n_out] = ord;
            sh->out[2 * sh->n_out + 1] = pm;
            sh->n_out++;
            continue;
        }
        sh->undo = (go_undo *)grow(sh->undo, &sh->cap_undo, sh->n_undo + 1, sizeof(go_undo));
        sh->undo[sh->n_undo].slot = slot;
        sh->undo[sh->n_undo].old = c->tab[slot];
        sh->n_undo++;
        apply_contact(c, pm, slot);
    }
}

static void shard_task(go_ctx *c, uint32_t tid, uint32_t nt) {
    (void)nt;
    c->sh[tid].n_undo = 0;
    c->sh[tid].n_used = 0;
    shard_run(c, tid);
}

/* reachability_unit, tracing/refinement.cpp:10-64: distance tests per
 * chunk, then the hash inserts and touches (:34-55) with the results of
 * applying them one at a time in test order */
static void stage_reachability(go_ctx *c) {
    const uint64_t B = c->cfg.num_meeting_buckets;
    go_parallel(c, gather_chunk);
    go_parallel(c, refine_chunk);
    c->contacts = 0;
    c->candidates = 0;
    for (uint32_t t = 0; t < c->threads; ++t) {
        c->candidates += c->tb[t].candidates;
        c->contacts += c->tb[t].n_contacts;
    }
    go_parallel(c, classify_chunk);
    go_parallel(c, touch_shard);
    go_parallel(c, shard_task);
    /* hand probes that ran off a range's end to the next range (the last
     * range's to the first: the probe wraps to slot 0) until no range's
     * entering probes change */
    const uint32_t T = c->threads;
    c->shard_rounds = 0;
    int changed = 1;
    for (uint32_t round = 0; changed; ++round) {
        changed = 0;
        for (uint32_t j = 0; j < T; ++j) {
            const go_shard *src = &c->sh[(j + T - 1) % T];
            go_shard *sh = &c->sh[j];
            if (src->n_out == sh->n_used && !memcmp(src->out, sh->used, 2 * sizeof(uint64_t) * src->n_out)) continue;
            sh->used = (uint64_t *)grow(sh->used, &sh->cap_used, 2 * src->n_out + 2, sizeof(uint64_t));
            memcpy(sh->used, src->out, 2 * sizeof(uint64_t) * src->n_out);
            sh->n_used = src->n_out;
            shard_run(c, j);
            c->shard_rounds++;
            changed = 1;
        }
        if (changed && round > 4 * T + 4) {
            /* no fixed point (a probe circling the whole table): undo every
             * range and apply the pairs one at a time */
            for (uint32_t j = 0; j < T; ++j) {
                go_shard *sh = &c->sh[j];
                while (sh->n_undo) { sh->n_undo--; c->tab[sh->undo[sh->n_undo].slot] = sh->undo[sh->n_undo].old; }
            }
            for (uint32_t t = 0; t < T; ++t) {
                /* merge every range's list of this chunk back into test order */
                size_t pos[GO_MAX_THREADS_SHARDS] = {0};
                for (;;) {
                    uint32_t best = T;
                    for (uint32_t j = 0; j < T; ++j)
                        if (pos[j] < c->tb[t].n_fresh[j] &&
                            (best == T || c->tb[t].fresh[j][2 * pos[j]] < c->tb[t].fresh[best][2 * pos[best]]))
                            best = j;
                    if (best == T) break;
                    uint64_t pm = c->tb[t].fresh[best][2 * pos[best] + 1];
                    apply_contact(c, pm, contact_slot(pm, B));
                    pos[best]++;
                }
            }
            break;
        }
    }
}

/* update_meetings_unit (tracing/meeting.cpp:32-76, batch_meet :11-24) over
 * one range of buckets; buckets are independent here */
static void identify_chunk(go_ctx *c, uint32_t tid, uint32_t nt) {
    size_t lo, hi;
    chunk_of(c->cfg.num_meeting_buckets, tid, nt, &lo, &hi);
    go_tbuf *tb = &c->tb[tid];
    tb->n_reports = 0;
    tb->taken = 0;
    tb->active = 0;
    for (size_t b = lo; b < hi; ++b) {
        go_rec *r = &c->tab[b];
        if (r->key == GO_EMPTY_KEY) continue;
        tb->taken++;
        if (r->end == c->cur_time) { tb->active++; continue; }
        if (c->cur_time - r->start >= c->cfg.min_meet_time + 1) {
            tb->reports = (go_meeting *)grow(tb->reports, &tb->cap_reports, tb->n_reports + 1, sizeof(go_meeting));
            go_meeting *m = &tb->reports[tb->n_reports++];
            m->key = r->key;
            m->start = r->start;
            m->end = r->end;
            memcpy(m->mbr, r->mbr, sizeof(m->mbr));
        }
        r->key = GO_EMPTY_KEY;
    }
}

/* update_meetings_unit, tracing/meeting.cpp:32-76: reports in bucket order */
static void stage_update_meetings(go_ctx *c) {
    go_parallel(c, identify_chunk);
    c->num_taken = 0;
    c->num_active = 0;
    uint64_t kv = 0;
    for (uint32_t t = 0; t < c->threads; ++t) {
        const go_tbuf *b = &c->tb[t];
        c->num_taken += b->taken;
        c->num_active += b->active;
        for (size_t i = 0; i < b->n_reports; ++i, ++kv)
            if (kv < c->cap_meetings) c->meetings[kv] = b->reports[i];
    }
    c->n_meetings = (uint32_t)kv;
}
/* workbench::merge_node, tracing/filter.cpp:316-336 */
static void merge_node(go_ctx *c, uint32_t cur) {
    c->n_merges++;
    for (int i = 0; i < 4; ++i) {
        uint32_t ch = c->schema[cur].children[i];
        c->schema[ch].type = GO_INVALID;
        c->schema_stack[--c->schema_stack_index] = ch;
        c->grids_stack[--c->grids_stack_index] = c->schema[ch].grid_id;
        c->grid_counter[c->schema[ch].grid_id] = 0;
    }
    c->schema[cur].type = GO_LEAF;
    c->schema[cur].grid_id = c->grids_stack[c->grids_stack_index++];
}

/* workbench::split_node, tracing/filter.cpp:338-375 */
static void split_node(go_ctx *c, uint32_t cur) {
    c->n_splits++;
    go_schema *p = &c->schema[cur];
    p->type = GO_BRANCH;
    c->grids_stack[--c->grids_stack_index] = p->grid_id;
    double xhalf = p->mid_x - p->low[0];
    double yhalf = p->mid_y - p->low[1];
    for (int i = 0; i < 4; ++i) {
        uint32_t child = c->schema_stack[c->schema_stack_index++];
        c->schema[cur].children[i] = child;
        go_schema *s = &c->schema[child];
        s->grid_id = c->grids_stack[c->grids_stack_index++];
        c->grid_counter[s->grid_id] = 0;
        s->level = c->schema[cur].level + 1;
        s->type = GO_LEAF;
        s->overflow_count = 0;
        s->underflow_count = 0;
        s->low[0] = c->schema[cur].low[0] + (i % 2 == 1) * xhalf;
        s->low[1] = c->schema[cur].low[1] + (i / 2 == 1) * yhalf;
        s->high[0] = c->schema[cur].mid_x + (i % 2 == 1) * xhalf;
        s->high[1] = c->schema[cur].mid_y + (i / 2 == 1) * yhalf;
        s->mid_x = (s->low[0] + s->high[0]) / 2;
        s->mid_y = (s->low[1] + s->high[1]) / 2;
    }
}

/* update_schema_unit, tracing/filter.cpp:377-424, over every schema slot in order */
static void stage_update_schema(go_ctx *c) {
    c->n_splits = 0;
    c->n_merges = 0;
    const double two_r = c->cfg.reach_distance * 2;
    for (uint32_t cur = 0; cur < c->schema_stack_capacity; ++cur) {
        go_schema *s = &c->schema[cur];
        if (s->type == GO_LEAF) {
            if (box_width_m(s->low, s->high) > two_r && c->grid_counter[s->grid_id] > c->cfg.grid_capacity) {
                s->overflow_count++;
                if ((uint32_t)s->overflow_count >= c->cfg.schema_update_delay) {
                    split_node(c, cur);
                    c->schema[cur].overflow_count = 0;
                }
            } else {
                s->overflow_count = 0;
            }
        } else if (s->type == GO_BRANCH) {
            int leafchild = 0;
            int ncounter = 0;
            for (int i = 0; i < 4; ++i) {
                uint32_t ch = s->children[i];
                if (c->schema[ch].type == GO_LEAF) {
                    leafchild++;
                    ncounter += c->grid_counter[c->schema[ch].grid_id];
                }
            }
            if (leafchild == 4 && ncounter < (int)c->cfg.grid_capacity) {
                s->underflow_count++;
                if ((uint32_t)s->underflow_count >= c->cfg.schema_update_delay) {
                    merge_node(c, cur);
                    c->schema[cur].underflow_count = 0;
                }
            } else {
                s->underflow_count = 0;
            }
        }
    }
}

int go_step(go_ctx *c, const double *points_xy, uint32_t cur_time) {
    /* workbench::reset, tracing/workbench.h:323-329 */
    memset(c->grid_counter, 0, sizeof(uint32_t) * c->grids_stack_capacity);
    c->pts = points_xy;
    c->cur_time = cur_time;
    stage_filter(c);
    stage_reachability(c);
    stage_update_meetings(c);
    if (c->cfg.dynamic_schema) stage_update_schema(c);
    c->pts = NULL;
    return 0;
}

void go_get_counts(const go_ctx *c, go_counts *o) {
    o->grid_check_counter = (uint32_t)c->n_checks;
    o->kv_count = c->n_meetings;
    o->num_taken_buckets = c->num_taken;
    o->num_active_meetings = c->num_active;
    o->grids_stack_index = c->grids_stack_index;
    o->schema_stack_index = c->schema_stack_index;
    o->grids_stack_capacity = c->grids_stack_capacity;
    o->schema_stack_capacity = c->schema_stack_capacity;
    o->grid_capacity = c->grid_capacity;
    o->contacts = c->contacts;
    o->candidates = c->candidates;
    o->n_splits = c->n_splits;
    o->n_merges = c->n_merges;
    o->x_buffer = c->x_buffer;
    o->y_buffer = c->y_buffer;
    o->range_reruns = c->shard_rounds;
    o->pad1 = 0;
}

uint32_t go_get_meetings(const go_ctx *c, go_meeting *out, uint32_t cap) {
    uint32_t n = c->n_meetings < c->cap_meetings ? c->n_meetings : c->cap_meetings;
    if (n > cap) n = cap;
    memcpy(out, c->meetings, sizeof(go_meeting) * n);
    return c->n_meetings;
}

void go_get_schema(const go_ctx *c, go_schema *schema, uint32_t *schema_stack, uint32_t *grids_stack,
                   uint32_t *grid_counter) {
    if (schema) memcpy(schema, c->schema, sizeof(go_schema) * c->schema_stack_capacity);
    if (schema_stack) memcpy(schema_stack, c->schema_stack, sizeof(uint32_t) * c->schema_stack_capacity);
    if (grids_stack) memcpy(grids_stack, c->grids_stack, sizeof(uint32_t) * c->grids_stack_capacity);
    if (grid_counter) memcpy(grid_counter, c->grid_counter, sizeof(uint32_t) * c->grids_stack_capacity);
}

void go_get_buckets(const go_ctx *c, uint64_t *keys, uint32_t *starts, uint32_t *ends, float *mbrs) {
    size_t B = c->cfg.num_meeting_buckets;
    for (size_t b = 0; b < B; ++b) {
        const go_rec *r = &c->tab[b];
        if (keys) keys[b] = r->key;
        if (starts) starts[b] = r->start;
        if (ends) ends[b] = r->end;
        if (mbrs) memcpy(mbrs + 4 * b, r->mbr, sizeof(float) * 4);
    }
}

/* The active multi-search of cuda_identify_meetings (cuda/geometry.cu:
 * 605-663) over the bucket table as it stands after the last step: a bucket
 * whose meeting is active (end == cur_time) and has lasted
 * cur_time - start >= min_meet_time + 1 yields one record per side whose id
 * is in the list, (listed id, other id, start, end, MBR).  The reference
 * appends with an atomic counter; here records come in bucket order, the
 * lower id's side first, and a repeated id in the list counts once. */
uint64_t go_active_search(const go_ctx *c, const uint32_t *pids, uint32_t npids, go_search_info *out,
                          uint64_t cap) {
    const uint32_t N = c->cfg.num_objects;
    uint8_t *in = (uint8_t *)calloc(N ? N : 1, 1);
    for (uint32_t i = 0; i < npids; ++i)
        if (pids[i] < N) in[pids[i]] = 1;
    uint64_t n = 0;
    const size_t B = c->cfg.num_meeting_buckets;
    for (size_t b = 0; b < B; ++b) {
        const go_rec *r = &c->tab[b];
        if (r->key == GO_EMPTY_KEY || r->end != c->cur_time) continue;
        if (c->cur_time - r->start < c->cfg.min_meet_time + 1) continue;
        uint32_t a, t;
        go_cantor_inverse(r->key, &a, &t);
        for (int side = 0; side < 2; ++side) {
            const uint32_t p = side ? t : a, q = side ? a : t;
            if (p >= N || !in[p]) continue;
            if (n < cap) {
                go_search_info *o = out + n;
                o->pid = p;
                o->target = q;
                o->start = r->start;
                o->end = r->end;
                memcpy(o->mbr, r->mbr, sizeof(float) * 4);
            }
            ++n;
        }
    }
    free(in);
    return n;
}
