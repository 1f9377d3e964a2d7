/*
 * fake_glint.c -- a CPU stand-in for the parts of libglint's C ABI
 * (include/glint.h) that the reference seam shim
 * (glint_pipeline_gb300/shim/glint_ref_shim.cpp) calls, built from the
 * oracle: go_step for the step, go_store for the flush into the key-value +
 * bitmap store, go_active_search for the searches.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets tests/test_shim.py run the reference's
 * own per-step loop and straight_dump through the shim on a machine without
 * a GPU, so that the shim's handoff (configuration, schema, stats, search
 * lists, the flushed block into the MemTable buffers, MemTable_count) is
 * checked by the reference's own consumer of it.  The step results of the
 * real library are checked against the same oracle by the GPU tests.
 *
 * The context is created at the first glint_step, from that step's points
 * (the first step is what the reference builds its schema from); the
 * schema the caller passed must equal the oracle's, or the step fails.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "glint.h"
#include "glint_oracle.h"

struct glint_ctx {
    glint_config cfg;
    double mbr[4];
    go_ctx *o;
    go_store *store;
    glint_schema_init init;
    glint_schema_node *init_nodes;
    uint32_t *init_sstack, *init_gstack;
    go_store_info info;
    int have_store;
    const char *err;
};

const char *glint_status_string(glint_status s) {
    switch (s) {
    case GLINT_OK: return "ok";
    case GLINT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GLINT_ERR_STATE: return "bad state";
    case GLINT_ERR_UNSUPPORTED: return "unsupported";
    default: return "error";
    }
}

const char *glint_last_error(const glint_ctx *c) { return c && c->err ? c->err : ""; }

void glint_config_defaults(glint_config *cfg, uint32_t n) {
    memset(cfg, 0, sizeof(*cfg));
    cfg->num_objects = n;
    cfg->grid_capacity = 50;
    cfg->grid_amplify = 2;
    cfg->num_meeting_buckets = 2ull * n;
    cfg->reach_distance = 2;
    cfg->min_meet_time = 5;
    cfg->max_meet_time = 4096;
    cfg->schema_update_delay = 1;
    cfg->dynamic_schema = 1;
    cfg->phased_lookup = 1;
    cfg->G_bytes = 2;
    cfg->CTF_count = 100;
    cfg->split_num = 10;
    cfg->dProbFalse = 100;
}

glint_status glint_host_alloc(size_t bytes, void **out) {
    *out = malloc(bytes ? bytes : 1);
    return *out ? GLINT_OK : GLINT_ERR_OUT_OF_MEMORY;
}

glint_status glint_host_free(void *p) {
    free(p);
    return GLINT_OK;
}

glint_status glint_create(const glint_config *cfg, const glint_box *mbr, const double *first_points,
                          const glint_schema_init *init, glint_ctx **out) {
    (void)first_points;
    glint_ctx *c = (glint_ctx *)calloc(1, sizeof(glint_ctx));
    c->cfg = *cfg;
    c->mbr[0] = mbr->low[0];
    c->mbr[1] = mbr->low[1];
    c->mbr[2] = mbr->high[0];
    c->mbr[3] = mbr->high[1];
    if (init) {
        c->init = *init;
        c->init_nodes = (glint_schema_node *)malloc(sizeof(glint_schema_node) * init->num_nodes);
        memcpy(c->init_nodes, init->nodes, sizeof(glint_schema_node) * init->num_nodes);
    }
    const uint64_t restriction = cfg->kv_restriction ? cfg->kv_restriction : (uint64_t)cfg->G_bytes << 25;
    const uint64_t extra = 4ull * cfg->num_objects > 1000000ull ? 4ull * cfg->num_objects : 1000000ull;
    c->cfg.kv_restriction = restriction;
    go_store_config sc;
    memset(&sc, 0, sizeof(sc));
    sc.num_objects = cfg->num_objects;
    sc.max_meet_time = cfg->max_meet_time;
    sc.CTF_count = cfg->CTF_count;
    sc.split_num = cfg->split_num;
    sc.first_end_time_min = cfg->start_time + cfg->min_meet_time;  /* tracing/process.cpp:404 */
    sc.dProbFalse = cfg->dProbFalse;
    memcpy(sc.mbr, c->mbr, sizeof(sc.mbr));
    sc.kv_capacity = cfg->kv_capacity ? cfg->kv_capacity : restriction + extra;
    c->store = go_store_create(&sc);
    *out = c;
    return GLINT_OK;
}

glint_status glint_destroy(glint_ctx *c) {
    if (!c) return GLINT_OK;
    go_destroy(c->o);
    go_store_destroy(c->store);
    free(c->init_nodes);
    free(c);
    return GLINT_OK;
}

/* the oracle's schema must be the one the caller built */
static int schema_matches(glint_ctx *c) {
    if (!c->init_nodes) return 1;
    go_counts k;
    go_get_counts(c->o, &k);
    if (k.schema_stack_index != c->init.schema_stack_index || k.grids_stack_index != c->init.grids_stack_index)
        return 0;
    go_schema *s = (go_schema *)malloc(sizeof(go_schema) * k.schema_stack_capacity);
    go_get_schema(c->o, s, NULL, NULL, NULL);
    int same = 1;
    for (uint32_t i = 0; i < k.schema_stack_index && i < c->init.num_nodes && same; ++i) {
        const glint_schema_node *g = &c->init_nodes[i];
        if (g->type != s[i].type || g->grid_id != s[i].grid_id || g->mid_x != s[i].mid_x || g->mid_y != s[i].mid_y)
            same = 0;
    }
    free(s);
    return same;
}

glint_status glint_step(glint_ctx *c, const double *points, uint32_t t, glint_step_stats *st) {
    if (!c->o) {
        go_config oc;
        memset(&oc, 0, sizeof(oc));
        oc.num_objects = c->cfg.num_objects;
        oc.grid_capacity = c->cfg.grid_capacity;
        oc.schema_update_delay = c->cfg.schema_update_delay;
        oc.min_meet_time = c->cfg.min_meet_time;
        oc.dynamic_schema = c->cfg.dynamic_schema;
        oc.num_meeting_buckets = c->cfg.num_meeting_buckets ? c->cfg.num_meeting_buckets : 2ull * oc.num_objects;
        oc.grid_amplify = c->cfg.grid_amplify;
        oc.reach_distance = c->cfg.reach_distance;
        c->o = go_create(&oc, c->mbr, points);
        if (!schema_matches(c)) {
            c->err = "the schema passed in differs from the oracle's build of the first step";
            return GLINT_ERR_STATE;
        }
    }
    go_step(c->o, points, t);
    go_counts k;
    go_get_counts(c->o, &k);
    memset(st, 0, sizeof(*st));
    st->cur_time = t;
    st->checks = k.grid_check_counter;
    st->candidates = k.candidates;
    st->contacts = k.contacts;
    st->num_taken_buckets = k.num_taken_buckets;
    st->num_active_meetings = k.num_active_meetings;
    st->meetings = k.kv_count;
    st->leaves = k.grids_stack_index;
    st->nodes = k.schema_stack_index;
    /* the step's meetings become keys (cuda_identify_meetings) */
    go_meeting *m = (go_meeting *)malloc(sizeof(go_meeting) * (k.kv_count ? k.kv_count : 1));
    uint32_t n = go_get_meetings(c->o, m, k.kv_count);
    go_meeting_rec *r = (go_meeting_rec *)malloc(sizeof(go_meeting_rec) * (n ? n : 1));
    for (uint32_t i = 0; i < n; ++i) {
        go_cantor_inverse(m[i].key, &r[i].pid1, &r[i].pid2);
        r[i].start = m[i].start;
        r[i].end = m[i].end;
        memcpy(r[i].mbr, m[i].mbr, sizeof(r[i].mbr));
    }
    go_store_add_meetings(c->store, r, n);
    free(m);
    free(r);
    st->kv_count = go_store_kv_count(c->store);
    if (c->cfg.auto_flush && st->kv_count > c->cfg.kv_restriction) {
        if (go_store_flush(c->store, t, &c->info) != 0) {
            c->err = "flush outside the reference's domain";
            return GLINT_ERR_UNSUPPORTED;
        }
        c->have_store = 1;
        st->flushed = 1;
        st->kv_count = go_store_kv_count(c->store);
    }
    return GLINT_OK;
}

glint_status glint_meetings(glint_ctx *c, glint_meeting *out, uint64_t cap, uint64_t *n) {
    go_counts k;
    go_get_counts(c->o, &k);
    *n = k.kv_count;
    if (!out || !cap) return GLINT_OK;
    go_meeting *m = (go_meeting *)malloc(sizeof(go_meeting) * (k.kv_count ? k.kv_count : 1));
    uint32_t got = go_get_meetings(c->o, m, k.kv_count);
    for (uint64_t i = 0; i < got && i < cap; ++i) {
        go_cantor_inverse(m[i].key, &out[i].pid1, &out[i].pid2);
        out[i].start = m[i].start;
        out[i].end = m[i].end;
        memcpy(out[i].mbr, m[i].mbr, sizeof(out[i].mbr));
    }
    free(m);
    return GLINT_OK;
}

glint_status glint_active_search(glint_ctx *c, const uint32_t *pids, uint32_t npids, glint_search_info *out,
                                 uint64_t cap, uint64_t *n) {
    _Static_assert(sizeof(glint_search_info) == sizeof(go_search_info), "search record layout");
    *n = go_active_search(c->o, pids, npids, (go_search_info *)out, out ? cap : 0);
    return GLINT_OK;
}

glint_status glint_store_read(glint_ctx *c, uint8_t *keys, uint16_t *sids, uint32_t *ctf_capacity,
                              glint_ctf_meta *ctfs, uint8_t *bitmaps, void *oversize_keys, float *oversize_boxes,
                              uint8_t *oversize_bitmap, glint_store_info *info) {
    _Static_assert(sizeof(glint_ctf_meta) == sizeof(go_ctf_meta), "CTF record layout");
    _Static_assert(sizeof(glint_store_info) == sizeof(go_store_info), "store info layout");
    if (!c->have_store) return GLINT_ERR_STATE;
    go_store_result(c->store, keys, sids, ctf_capacity, (go_ctf_meta *)ctfs, bitmaps, oversize_keys,
                    oversize_boxes, oversize_bitmap);
    if (info) memcpy(info, &c->info, sizeof(*info));
    return GLINT_OK;
}
