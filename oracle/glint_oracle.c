/*
 * glint_oracle.c -- single-threaded CPU restatement of the reference's
 * per-timestep contact-tracing stages.  TEST ORACLE ONLY: imported by tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline leg, never by the
 * product path.  Build: oracle/Makefile (gcc -O2 -ffp-contract=off).
 *
 * Every function names the reference lines it follows.  Where the reference
 * runs a stage on several pthreads, this file runs it on one thread in the
 * reference's batch order, which is the only order in which the reference's
 * results are reproducible (leaf-overflow drops and hash-slot placement depend
 * on it).
 */
#include "glint_oracle.h"

#include <math.h>
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
    uint32_t *grid_counter;
    uint32_t *grids_stack;
    uint32_t *schema_stack;
    go_schema *schema;

    go_check *checks;
    size_t n_checks, cap_checks;

    uint64_t *bkey;
    uint32_t *bstart, *bend;
    float *bmbr;                       /* [B*4] */

    go_meeting *meetings;              /* identified in the last step */
    uint32_t n_meetings, cap_meetings;
    uint64_t num_taken;
    uint32_t num_active;
    uint64_t contacts, candidates;
    uint32_t n_splits, n_merges;
};

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

/* Point::distance(p, true), geometry/geometry.h:40-48; p1 is the caller */
static double point_distance(double x1, double y1, double x2, double y2) {
    double dx = x1 - x2;
    double dy = y1 - y2;
    dy = dy / go_dpm_lat_c;
    dx = dx / go_dpm_lon(y1);
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

go_ctx *go_create(const go_config *cfg, const double *mbr4, const double *points_xy) {
    go_ctx *c = (go_ctx *)calloc(1, sizeof(go_ctx));
    c->cfg = *cfg;
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
    c->grids_stack = (uint32_t *)malloc(sizeof(uint32_t) * c->grids_stack_capacity);
    for (uint32_t i = 0; i < c->grids_stack_capacity; ++i) c->grids_stack[i] = i;
    c->schema = (go_schema *)calloc(c->schema_stack_capacity, sizeof(go_schema));
    c->schema_stack = (uint32_t *)malloc(sizeof(uint32_t) * c->schema_stack_capacity);
    for (uint32_t i = 0; i < c->schema_stack_capacity; ++i) {
        c->schema_stack[i] = i;
        c->schema[i].type = GO_INVALID;
    }
    size_t B = cfg->num_meeting_buckets;
    c->bkey = (uint64_t *)malloc(sizeof(uint64_t) * B);
    c->bstart = (uint32_t *)calloc(B, sizeof(uint32_t));
    c->bend = (uint32_t *)calloc(B, sizeof(uint32_t));
    c->bmbr = (float *)calloc(B * 4, sizeof(float));
    for (size_t i = 0; i < B; ++i) c->bkey[i] = GO_EMPTY_KEY;
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
    free(c->grids); free(c->grid_counter); free(c->grids_stack); free(c->schema); free(c->schema_stack);
    free(c->checks); free(c->bkey); free(c->bstart); free(c->bend); free(c->bmbr); free(c->meetings);
    free(c);
}

static void push_check(go_ctx *c, uint32_t pid, uint32_t gid, uint32_t inside) {
    if (c->n_checks == c->cap_checks) {
        c->cap_checks *= 2;
        c->checks = (go_check *)realloc(c->checks, sizeof(go_check) * c->cap_checks);
    }
    go_check *k = &c->checks[c->n_checks++];
    k->pid = pid; k->gid = gid; k->inside = inside;
}

/* lookup_rec, tracing/filter.cpp:130-152 (query_all == false) */
static void lookup_rec(go_ctx *c, double px, double py, uint32_t pid, uint32_t curnode) {
    for (int i = 0; i < 4; ++i) {
        uint32_t child = c->schema[curnode].children[i];
        const go_schema *s = &c->schema[child];
        double dist = box_distance(s, px, py);
        if (dist <= c->cfg.reach_distance) {
            if (s->type == GO_LEAF) {
                if (py < s->low[1] || (py < s->high[1] && px < s->low[0]))
                    push_check(c, pid, s->grid_id, 0);
            } else {
                lookup_rec(c, px, py, pid, child);
            }
        }
    }
}

/* workbench::filter + filter_unit (phased), tracing/filter.cpp:209-313 */
static void stage_filter(go_ctx *c) {
    uint32_t n = c->cfg.num_objects;
    c->n_checks = n;                              /* grid_check_counter = N */
    if (c->cap_checks < n) {
        c->cap_checks = (size_t)n * 2;
        c->checks = (go_check *)realloc(c->checks, sizeof(go_check) * c->cap_checks);
    }
    for (uint32_t pid = 0; pid < n; ++pid) {
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
        /* workbench::insert, tracing/filter.cpp:95-111 */
        uint32_t gid = c->schema[curnode].grid_id;
        uint32_t cur_size = c->grid_counter[gid]++;
        if (cur_size < c->grid_capacity) c->grids[(size_t)c->grid_capacity * gid + cur_size] = pid;
        c->checks[pid].pid = pid;
        c->checks[pid].gid = gid;
        c->checks[pid].inside = 1;
        if (last_valid != curnode) lookup_rec(c, px, py, pid, last_valid);
    }
}

static void mbr_update_by_point(float *m, double x, double y) { /* cuda/geometry.cu:82-96 */
    if (m[0] > x) m[0] = (float)x;
    if (m[2] < x) m[2] = (float)x;
    if (m[1] > y) m[1] = (float)y;
    if (m[3] < y) m[3] = (float)y;
}

/* reachability_unit, tracing/refinement.cpp:10-64 */
static void stage_reachability(go_ctx *c) {
    const uint64_t B = c->cfg.num_meeting_buckets;
    c->contacts = 0;
    c->candidates = 0;
    for (size_t k = 0; k < c->n_checks; ++k) {
        uint32_t pid = c->checks[k].pid, gid = c->checks[k].gid;
        uint32_t size = c->grid_counter[gid] < c->grid_capacity ? c->grid_counter[gid] : c->grid_capacity;
        const uint32_t *members = c->grids + (size_t)c->grid_capacity * gid;
        double x1 = pt_x(c, pid), y1 = pt_y(c, pid);
        for (uint32_t i = 0; i < size; ++i) {
            uint32_t m = members[i];
            if (!(pid < m || !c->checks[k].inside)) continue;
            c->candidates++;
            double x2 = pt_x(c, m), y2 = pt_y(c, m);
            if (point_distance(x1, y1, x2, y2) <= c->cfg.reach_distance) {
                c->contacts++;
                uint32_t p1 = pid < m ? pid : m;
                uint32_t p2 = pid < m ? m : pid;
                uint64_t key = go_cantor(p1, p2);
                uint64_t slot = key % B;
                for (;;) {
                    if (c->bkey[slot] == key) {
                        c->bend[slot] = c->cur_time;
                        mbr_update_by_point(&c->bmbr[4 * slot], x1, y1);
                        mbr_update_by_point(&c->bmbr[4 * slot], x2, y2);
                        break;
                    } else if (c->bkey[slot] == GO_EMPTY_KEY) {
                        c->bkey[slot] = key;
                        c->bstart[slot] = c->cur_time;
                        c->bend[slot] = c->cur_time;
                        float *mb = &c->bmbr[4 * slot];
                        mb[0] = 100000.0f; mb[1] = 100000.0f; mb[2] = -100000.0f; mb[3] = -100000.0f;
                        mbr_update_by_point(mb, x1, y1);
                        mbr_update_by_point(mb, x2, y2);
                        break;
                    }
                    slot = (slot + 1) % B;
                }
            }
        }
    }
}

/* update_meetings_unit, tracing/meeting.cpp:32-76 and batch_meet :11-24 */
static void stage_update_meetings(go_ctx *c) {
    const uint64_t B = c->cfg.num_meeting_buckets;
    c->n_meetings = 0;
    c->num_taken = 0;
    c->num_active = 0;
    uint32_t kv = 0;
    for (uint64_t b = 0; b < B; ++b) {
        if (c->bkey[b] == GO_EMPTY_KEY) continue;
        c->num_taken++;
        if (c->bend[b] == c->cur_time) { c->num_active++; continue; }
        if (c->cur_time - c->bstart[b] >= c->cfg.min_meet_time + 1) {
            if (kv < c->cap_meetings) {
                go_meeting *m = &c->meetings[kv];
                m->key = c->bkey[b];
                m->start = c->bstart[b];
                m->end = c->bend[b];
                memcpy(m->mbr, &c->bmbr[4 * b], sizeof(m->mbr));
            }
            kv++;
        }
        c->bkey[b] = GO_EMPTY_KEY;
    }
    c->n_meetings = kv;
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
    if (keys) memcpy(keys, c->bkey, sizeof(uint64_t) * B);
    if (starts) memcpy(starts, c->bstart, sizeof(uint32_t) * B);
    if (ends) memcpy(ends, c->bend, sizeof(uint32_t) * B);
    if (mbrs) memcpy(mbrs, c->bmbr, sizeof(float) * 4 * B);
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
        if (c->bkey[b] == GO_EMPTY_KEY || c->bend[b] != c->cur_time) continue;
        if (c->cur_time - c->bstart[b] < c->cfg.min_meet_time + 1) continue;
        uint32_t a, t;
        go_cantor_inverse(c->bkey[b], &a, &t);
        for (int side = 0; side < 2; ++side) {
            const uint32_t p = side ? t : a, q = side ? a : t;
            if (p >= N || !in[p]) continue;
            if (n < cap) {
                go_search_info *o = out + n;
                o->pid = p;
                o->target = q;
                o->start = c->bstart[b];
                o->end = c->bend[b];
                memcpy(o->mbr, c->bmbr + 4 * b, sizeof(float) * 4);
            }
            ++n;
        }
    }
    free(in);
    return n;
}
