/*
 * tracegen.h -- seeded synthetic Manhattan-grid trajectories.
 *
 * Stand-in for the reference's trace input (timestep-major Point arrays, one
 * FP64 lon/lat pair per object per 1 s step: tracing/process.cpp:128-144,
 * tracing/process.cpp:434, tools/datagen.cpp:18-26).  The reference's own
 * generator (tracing/generator.cpp:387-406) walks a Chicago street graph and
 * seeds from the wall clock, so it is not reproducible; this generator is.
 *
 * Model: a square box of `extent_m` metres with streets every `block_m`
 * metres in both directions.  Objects start at Gaussian hotspots or uniformly,
 * snapped to the nearest street, and walk along streets at U(speed_min,
 * speed_max) m/s; a fraction never moves.  At an intersection an object picks
 * uniformly among the directions that stay inside the box.
 *
 * Determinism: every value comes from a counter-based hash of
 * (seed, object, step, draw) and only IEEE add/sub/mul/div/floor/round, so the
 * host build (compiled with -ffp-contract=off) and the CUDA build (explicit
 * _rn intrinsics, no contraction) produce bit-identical coordinates on x86-64
 * and aarch64.  Gaussian offsets use the Irwin-Hall sum of 12 uniforms minus
 * 6 (unit variance, support +-6 sigma), which needs no transcendental.
 *
 * Metres map to degrees with fixed constants: the latitude factor is
 * 360/(40076*1000) (util/util.h:57) and the longitude factor is the
 * reference's degree_per_meter_longitude(41.6) (util/util.h:59-66) evaluated
 * once and written below as an exact hex literal, so no libm call is needed.
 */
#ifndef GLINT_TRACEGEN_H_
#define GLINT_TRACEGEN_H_

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define TG_FN __host__ __device__ static inline
#else
#define TG_FN static inline
#endif

/* exact-rounding arithmetic that no compiler may fuse */
#if defined(__CUDA_ARCH__)
#define TG_ADD(a, b) __dadd_rn((a), (b))
#define TG_SUB(a, b) __dsub_rn((a), (b))
#define TG_MUL(a, b) __dmul_rn((a), (b))
#define TG_DIV(a, b) __ddiv_rn((a), (b))
#else
#define TG_ADD(a, b) ((a) + (b))
#define TG_SUB(a, b) ((a) - (b))
#define TG_MUL(a, b) ((a) * (b))
#define TG_DIV(a, b) ((a) / (b))
#endif

#define TG_MAX_HOTSPOTS 64

/* degree_per_meter_longitude(41.6) with the reference's formula and glibc sin */
#define TG_DPM_LON_41_6 0x1.9312ae031405fp-17
/* 360.0/(40076.0*1000.0) */
#define TG_DPM_LAT 0x1.2d6acd5025901p-17

typedef struct tg_params {
    uint64_t seed;
    uint32_t num_objects;
    uint32_t n_hotspots;
    double origin_lon;      /* lon of the box's west edge */
    double origin_lat;      /* lat of the box's south edge */
    double deg_per_m_lon;
    double deg_per_m_lat;
    double extent_m;        /* box side, metres */
    double block_m;         /* street spacing, metres */
    double sigma_m;         /* hotspot standard deviation, metres */
    double hotspot_frac;    /* fraction of objects that start at a hotspot */
    double stationary_frac;
    double speed_min;
    double speed_max;
    double hotspot_x[TG_MAX_HOTSPOTS];
    double hotspot_y[TG_MAX_HOTSPOTS];
} tg_params;

/* one object: on the street segment from lower grid point `ga` (index along
 * the moving axis) at perpendicular street index `gb`, offset `u` metres */
typedef struct tg_object {
    double u;
    double speed;
    int32_t ga;
    int32_t gb;
    uint32_t flags;         /* bit0 axis (0: moves along x), bit1 dir (1: negative), bit2 stationary */
    uint32_t pad;
} tg_object;

#define TG_AXIS_Y 1u
#define TG_DIR_NEG 2u
#define TG_STATIONARY 4u

TG_FN uint64_t tg_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* uniform double in [0,1) keyed by (seed, stream, counter) */
TG_FN double tg_uniform(uint64_t seed, uint64_t stream, uint64_t counter) {
    uint64_t z = tg_mix64(seed ^ tg_mix64(stream * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL)
                          ^ (counter * 0xD1B54A32D192ED03ULL));
    return (double)(z >> 11) * 0x1.0p-53;
}

TG_FN double tg_gauss12(uint64_t seed, uint64_t stream, uint64_t counter0) {
    double s = 0.0;
    for (int k = 0; k < 12; ++k) s = TG_ADD(s, tg_uniform(seed, stream, counter0 + (uint64_t)k));
    return TG_SUB(s, 6.0);
}

/* streams: objects use stream oid+1; hotspot centres use stream 0 */
#define TG_INIT_COUNTER 0x100000000ULL

/* default Manhattan box: lon/lat origin (-88.0, 41.6), 40x40 km, 100 m blocks */
TG_FN void tg_default_params(tg_params *p, uint64_t seed, uint32_t n) {
    p->seed = seed;
    p->num_objects = n;
    p->n_hotspots = 8;
    p->origin_lon = -88.0;
    p->origin_lat = 41.6;
    p->deg_per_m_lon = TG_DPM_LON_41_6;
    p->deg_per_m_lat = TG_DPM_LAT;
    p->extent_m = 40000.0;
    p->block_m = 100.0;
    p->sigma_m = 500.0;
    p->hotspot_frac = 0.7;
    p->stationary_frac = 0.1;
    p->speed_min = 0.5;
    p->speed_max = 2.0;
    for (int i = 0; i < TG_MAX_HOTSPOTS; ++i) { p->hotspot_x[i] = 0.0; p->hotspot_y[i] = 0.0; }
}

/* place hotspot centres (call after editing n_hotspots / sigma / extent) */
TG_FN void tg_place_hotspots(tg_params *p) {
    double margin = TG_MUL(3.0, p->sigma_m);
    double span = TG_SUB(p->extent_m, TG_MUL(2.0, margin));
    if (span < 0.0) { margin = 0.0; span = p->extent_m; }
    for (uint32_t h = 0; h < p->n_hotspots && h < TG_MAX_HOTSPOTS; ++h) {
        p->hotspot_x[h] = TG_ADD(margin, TG_MUL(span, tg_uniform(p->seed, 0, 2 * (uint64_t)h)));
        p->hotspot_y[h] = TG_ADD(margin, TG_MUL(span, tg_uniform(p->seed, 0, 2 * (uint64_t)h + 1)));
    }
}

TG_FN double tg_clamp(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

TG_FN void tg_init_object(const tg_params *p, uint32_t oid, tg_object *o) {
    const uint64_t st = (uint64_t)oid + 1;
    const uint64_t c = TG_INIT_COUNTER;
    double px, py;
    if (tg_uniform(p->seed, st, c + 0) < p->hotspot_frac && p->n_hotspots > 0) {
        uint32_t h = (uint32_t)TG_MUL(tg_uniform(p->seed, st, c + 1), (double)p->n_hotspots);
        if (h >= p->n_hotspots) h = p->n_hotspots - 1;
        px = TG_ADD(p->hotspot_x[h], TG_MUL(p->sigma_m, tg_gauss12(p->seed, st, c + 16)));
        py = TG_ADD(p->hotspot_y[h], TG_MUL(p->sigma_m, tg_gauss12(p->seed, st, c + 32)));
    } else {
        px = TG_MUL(p->extent_m, tg_uniform(p->seed, st, c + 2));
        py = TG_MUL(p->extent_m, tg_uniform(p->seed, st, c + 3));
    }
    px = tg_clamp(px, 0.0, p->extent_m);
    py = tg_clamp(py, 0.0, p->extent_m);
    const double B = p->block_m;
    const int32_t nb = (int32_t)TG_DIV(p->extent_m, B); /* blocks per side */
    double rx = round(TG_DIV(px, B)), ry = round(TG_DIV(py, B));
    double dx = fabs(TG_SUB(px, TG_MUL(rx, B)));
    double dy = fabs(TG_SUB(py, TG_MUL(ry, B)));
    uint32_t flags = 0;
    double along, u;
    int32_t ga, gb;
    if (dy <= dx) {            /* snap onto the horizontal street y = ry*B, move along x */
        gb = (int32_t)ry;
        along = px;
    } else {                   /* vertical street x = rx*B, move along y */
        gb = (int32_t)rx;
        along = py;
        flags |= TG_AXIS_Y;
    }
    ga = (int32_t)floor(TG_DIV(along, B));
    if (ga < 0) ga = 0;
    if (ga > nb - 1) ga = nb - 1;
    u = tg_clamp(TG_SUB(along, TG_MUL((double)ga, B)), 0.0, B);
    if (tg_uniform(p->seed, st, c + 4) < 0.5) flags |= TG_DIR_NEG;
    if (tg_uniform(p->seed, st, c + 5) < p->stationary_frac) flags |= TG_STATIONARY;
    o->u = u;
    o->speed = TG_ADD(p->speed_min, TG_MUL(TG_SUB(p->speed_max, p->speed_min), tg_uniform(p->seed, st, c + 6)));
    o->ga = ga;
    o->gb = gb;
    o->flags = flags;
    o->pad = 0;
}

/* at grid point (X, Y) pick a direction that stays inside the box and set
 * the object onto that segment at the intersection */
TG_FN void tg_turn(const tg_params *p, tg_object *o, int32_t X, int32_t Y, uint32_t oid, uint32_t t, uint32_t k) {
    const int32_t nb = (int32_t)TG_DIV(p->extent_m, p->block_m);
    int dirs[4];
    int nd = 0;
    if (X < nb) dirs[nd++] = 0; /* +x */
    if (X > 0) dirs[nd++] = 1;  /* -x */
    if (Y < nb) dirs[nd++] = 2; /* +y */
    if (Y > 0) dirs[nd++] = 3;  /* -y */
    double uu = tg_uniform(p->seed, (uint64_t)oid + 1, (uint64_t)t * 4 + k);
    int pick = (int)TG_MUL(uu, (double)nd);
    if (pick >= nd) pick = nd - 1;
    uint32_t stat = o->flags & TG_STATIONARY;
    switch (dirs[pick]) {
    case 0: o->flags = stat;                         o->ga = X;     o->gb = Y; o->u = 0.0;          break;
    case 1: o->flags = stat | TG_DIR_NEG;            o->ga = X - 1; o->gb = Y; o->u = p->block_m;   break;
    case 2: o->flags = stat | TG_AXIS_Y;             o->ga = Y;     o->gb = X; o->u = 0.0;          break;
    default: o->flags = stat | TG_AXIS_Y | TG_DIR_NEG; o->ga = Y - 1; o->gb = X; o->u = p->block_m; break;
    }
}

/* advance one object by one 1-second step (t = index of the step being produced) */
TG_FN void tg_advance(const tg_params *p, tg_object *o, uint32_t oid, uint32_t t) {
    if (o->flags & TG_STATIONARY) return;
    double rem = o->speed;
    const double B = p->block_m;
    for (uint32_t k = 0; k < 3 && rem > 0.0; ++k) {
        int neg = (o->flags & TG_DIR_NEG) != 0;
        double d = neg ? o->u : TG_SUB(B, o->u);
        if (rem < d) {
            o->u = neg ? TG_SUB(o->u, rem) : TG_ADD(o->u, rem);
            rem = 0.0;
        } else {
            rem = TG_SUB(rem, d);
            int32_t a = neg ? o->ga : o->ga + 1; /* grid index of the intersection along the axis */
            int32_t X, Y;
            if (o->flags & TG_AXIS_Y) { X = o->gb; Y = a; } else { X = a; Y = o->gb; }
            tg_turn(p, o, X, Y, oid, t, k);
        }
    }
}

/* lon/lat of an object */
TG_FN void tg_position(const tg_params *p, const tg_object *o, double *lon, double *lat) {
    const double B = p->block_m;
    double along = TG_ADD(TG_MUL((double)o->ga, B), o->u);
    double perp = TG_MUL((double)o->gb, B);
    double xm = (o->flags & TG_AXIS_Y) ? perp : along;
    double ym = (o->flags & TG_AXIS_Y) ? along : perp;
    *lon = TG_ADD(p->origin_lon, TG_MUL(xm, p->deg_per_m_lon));
    *lat = TG_ADD(p->origin_lat, TG_MUL(ym, p->deg_per_m_lat));
}

/* the map box that contains every generated point */
TG_FN void tg_map_box(const tg_params *p, double *low_lon, double *low_lat, double *high_lon, double *high_lat) {
    *low_lon = p->origin_lon;
    *low_lat = p->origin_lat;
    *high_lon = TG_ADD(p->origin_lon, TG_MUL(p->extent_m, p->deg_per_m_lon));
    *high_lat = TG_ADD(p->origin_lat, TG_MUL(p->extent_m, p->deg_per_m_lat));
}

#endif /* GLINT_TRACEGEN_H_ */
