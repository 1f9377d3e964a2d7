/*
 * tracegen_host.c -- host entry points of the synthetic trajectory generator
 * (tracegen.h).  Built with -ffp-contract=off so every coordinate is the same
 * bit pattern as the device generator's.
 *
 * Output layout matches the reference's trace buffers: timestep-major, one
 * (lon, lat) FP64 pair per object (tracing/process.cpp:434,
 * tools/datagen.cpp:18-26).
 */
#include "tracegen.h"
#include <stdlib.h>
#include <string.h>

typedef struct tg_state {
    tg_params params;
    tg_object *objects;
    uint32_t step;          /* index of the next step to be produced */
} tg_state;

/* configure a generator; `kind` 0 = Manhattan box with 8 hotspots (sigma 500 m,
 * 70% of objects); 1 = extreme skew (5 hotspots, sigma 50 m, 20%) */
tg_state *tg_create(uint64_t seed, uint32_t n, int kind) {
    tg_state *s = (tg_state *)calloc(1, sizeof(tg_state));
    if (!s) return NULL;
    tg_default_params(&s->params, seed, n);
    if (kind == 1) {
        s->params.n_hotspots = 5;
        s->params.sigma_m = 50.0;
        s->params.hotspot_frac = 0.2;
    }
    tg_place_hotspots(&s->params);
    s->objects = (tg_object *)malloc(sizeof(tg_object) * (size_t)(n ? n : 1));
    if (!s->objects) { free(s); return NULL; }
    for (uint32_t i = 0; i < n; ++i) tg_init_object(&s->params, i, &s->objects[i]);
    s->step = 0;
    return s;
}

/* override box/hotspot parameters before the first step (re-initialises objects) */
void tg_set_shape(tg_state *s, double extent_m, double block_m, uint32_t n_hotspots, double sigma_m,
                  double hotspot_frac, double stationary_frac) {
    s->params.extent_m = extent_m;
    s->params.block_m = block_m;
    s->params.n_hotspots = n_hotspots > TG_MAX_HOTSPOTS ? TG_MAX_HOTSPOTS : n_hotspots;
    s->params.sigma_m = sigma_m;
    s->params.hotspot_frac = hotspot_frac;
    s->params.stationary_frac = stationary_frac;
    tg_place_hotspots(&s->params);
    for (uint32_t i = 0; i < s->params.num_objects; ++i) tg_init_object(&s->params, i, &s->objects[i]);
    s->step = 0;
}

/* produce `nsteps` consecutive steps into out[nsteps][n][2] */
void tg_generate(tg_state *s, uint32_t nsteps, double *out) {
    const uint32_t n = s->params.num_objects;
    for (uint32_t k = 0; k < nsteps; ++k) {
        if (s->step > 0)
            for (uint32_t i = 0; i < n; ++i) tg_advance(&s->params, &s->objects[i], i, s->step);
        double *o = out + (size_t)k * n * 2;
        for (uint32_t i = 0; i < n; ++i) tg_position(&s->params, &s->objects[i], &o[2 * i], &o[2 * i + 1]);
        s->step++;
    }
}

void tg_box(const tg_state *s, double *out4) {
    tg_map_box(&s->params, &out4[0], &out4[1], &out4[2], &out4[3]);
}

/* raw parameter block and object states, for the device generator */
const tg_params *tg_get_params(const tg_state *s) { return &s->params; }
uint32_t tg_params_size(void) { return (uint32_t)sizeof(tg_params); }
uint32_t tg_object_size(void) { return (uint32_t)sizeof(tg_object); }
void tg_get_objects(const tg_state *s, void *out) {
    memcpy(out, s->objects, sizeof(tg_object) * (size_t)s->params.num_objects);
}
uint32_t tg_current_step(const tg_state *s) { return s->step; }

void tg_destroy(tg_state *s) {
    if (!s) return;
    free(s->objects);
    free(s);
}
