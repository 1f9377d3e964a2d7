/*
 * glint_device.cuh -- device-side types and exact-arithmetic helpers shared by
 * the per-step kernels.
 *
 * Exactness contract: every FP64 expression the reference evaluates on the
 * host (compiled without FMA contraction) is evaluated here with explicit
 * _rn intrinsics in the same order, so the rounded results are identical.
 * The one libm call in the path, sin() inside degree_per_meter_longitude
 * (util/util.h:59-66), is evaluated with CUDA's sin for speed; any decision
 * whose outcome could change under the last-bit differences between that and
 * the host libm is re-taken with a correctly rounded double-double sin and
 * its two neighbouring doubles (see dist_le_exact below).
 */
#ifndef GLINT_DEVICE_CUH_
#define GLINT_DEVICE_CUH_

#include <cstdint>
#include <cuda_runtime.h>

#include "glint_types.h"

namespace glint {

/* ---- constants (util/util.h:38-39, 57) --------------------------------- */
constexpr double kPI = 3.14159265;
constexpr uint64_t kEmptyKey = 1ULL << 62;           /* ULL_MAX */
constexpr uint64_t kNewFlag = 1ULL << 63;            /* key inserted during this step */
constexpr uint64_t kKeyMask = (1ULL << 62) - 1;

enum : uint8_t { kInvalid = 0, kBranch = 1, kLeaf = 2 }; /* index/QTree.h:43-47 */

/* stamp byte per table slot: 0 empty (or filled during the current step), 1
 * committed entry (4: reported this step, identify only).  Which step last
 * touched a committed entry is its tag, 1 or 2 by step parity, in the high
 * half of the record's w1 (the low half holds the start time), so a touch
 * writes only the record it has just read.  A slot filled during the step
 * carries kNewFlag in its key word; the insert marks its 128-byte line (four
 * slots) in a bitmap small enough to stay in L2 instead of writing a stamp
 * byte, which would cost a random DRAM read-modify-write per new pair. */
enum : uint8_t { kStampEmpty = 0, kStampOld = 1 };
__host__ __device__ inline uint8_t stamp_of(uint64_t step_index) { return (uint8_t)(1 + (step_index & 1)); }

/* ---- exact comparisons without the FP64 pipe --------------------------------
 * On sm_103a every FP64 instruction, compares and conversions included, issues
 * at a small fraction of the FP32 rate, so the hot loops compare doubles as
 * order-preserving 64-bit keys: for non-NaN doubles a < b exactly when
 * dkey(a) < dkey(b) (-0 is folded onto +0, which IEEE compares equal). */
__host__ __device__ inline uint64_t dbits(double d) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    memcpy(&b, &d, 8);
    return b;
#endif
}
__host__ __device__ inline double bitsd(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}
__host__ __device__ inline uint64_t dkey(double d) {
    uint64_t b = dbits(d);
    if (b == 0x8000000000000000ull) b = 0;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double kdbl(uint64_t k) {
    return bitsd((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k);
}

/* ---- schema node as stored on the device (64 bytes, one half line) ----
 * The reference's QTSchema (index/QTree.h:49-62) is 80 bytes with the low
 * corner in the middle; the descent only needs mid, high, children and type,
 * so those share one 64-byte record (as comparison keys) and the low corner
 * lives beside it. */
struct __align__(64) DNode {
    uint64_t kmx, kmy;   /* dkey(mid_x), dkey(mid_y) */
    uint64_t khx, khy;   /* dkey(high_x), dkey(high_y) */
    uint32_t child[4];
    uint32_t gid;
    uint8_t type;
    uint8_t pad0;
    int16_t level;
    int16_t of;          /* overflow_count */
    int16_t uf;          /* underflow_count */
    uint32_t pad1;
};
static_assert(sizeof(DNode) == 64, "DNode must be 64 bytes");

/* ---- meeting-table record (32 bytes, one sector) ----
 * The bucket of a pair (a < b) is cantorPairing(a, b) % B as in the
 * reference (tracing/refinement.cpp:34-37); the record stores the pair itself
 * instead of the Cantor key, which is equivalent and needs no inverse.
 * w0: (a << 32) | b (committed), kNewFlag | (a << 32) | b (inserted this
 *     step) or kEmptyW0
 * w1: (touch tag << 32) | start time (committed) or insertion priority (new)
 * mbr: order-preserving encodings of the f32 box (low x, low y, high x, high y) */
struct __align__(32) TRec {
    unsigned long long w0;
    unsigned long long w1;
    uint32_t mbr[4];
};
static_assert(sizeof(TRec) == 32, "TRec must be 32 bytes");
constexpr unsigned long long kEmptyW0 = ~0ull;
constexpr unsigned long long kPairMask = ~kNewFlag;

/* the touch tag of a committed record */
__device__ inline uint32_t rec_tag(const TRec &r) { return (uint32_t)(r.w1 >> 32); }
__device__ inline void rec_set_tag(TRec &r, uint32_t tag) { reinterpret_cast<uint32_t *>(&r.w1)[1] = tag; }

__host__ __device__ inline unsigned long long pair_word(uint32_t a, uint32_t b) {
    return ((unsigned long long)a << 32) | b;
}
__host__ __device__ inline uint32_t pair_a(unsigned long long w) { return (uint32_t)(w >> 32) & 0x7fffffffu; }
__host__ __device__ inline uint32_t pair_b(unsigned long long w) { return (uint32_t)w; }

__host__ __device__ inline uint32_t fenc(float f) {
    uint32_t u;
#if defined(__CUDA_ARCH__)
    u = __float_as_uint(f);
#else
    memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float fdec(uint32_t e) {
    uint32_t u = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

/* ---- Cantor pairing (util/util.h:68-70) and its exact inverse ---------- */
__host__ __device__ inline uint64_t cantor(uint32_t a, uint32_t b) {
    return (uint64_t)(a + b) * (a + b + 1) / 2 + b;
}
__device__ inline void cantor_inverse(uint64_t z, uint32_t &a, uint32_t &b) {
    uint64_t w = (uint64_t)floor((sqrt(8.0 * (double)z + 1.0) - 1.0) * 0.5);
    while (w > 0 && w * (w + 1) / 2 > z) --w;
    while ((w + 1) * (w + 2) / 2 <= z) ++w;
    uint64_t t = w * (w + 1) / 2;
    b = (uint32_t)(z - t);
    a = (uint32_t)(w - b);
}

/* z mod B with a precomputed m = floor((2^64-1)/B): q = mulhi(z, m) is
 * floor(z/B) or one less */
__device__ inline uint64_t fastmod(uint64_t z, uint64_t B, uint64_t m) {
    uint64_t q = __umul64hi(z, m);
    uint64_t r = z - q * B;
    return r >= B ? r - B : r;
}

/* ---- double-double sin, correctly rounded on [0, pi/2] -------------------
 * Horner evaluation of the Taylor series to x^41/41! in double-double
 * arithmetic (Dekker/Knuth two-sum, fma two-product).  The coefficients
 * (-1)^k/(2k+1)! are computed in double-double at context creation. */
struct DD { double hi, lo; };

__device__ inline DD dd_quick(double a, double b) {
    double s = __dadd_rn(a, b);
    return DD{s, __dsub_rn(b, __dsub_rn(s, a))};
}
__device__ inline DD dd_two_sum(double a, double b) {
    double s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
    return DD{s, e};
}
__device__ inline DD dd_add(DD a, DD b) {
    DD s = dd_two_sum(a.hi, b.hi);
    DD t = dd_two_sum(a.lo, b.lo);
    s.lo = __dadd_rn(s.lo, t.hi);
    s = dd_quick(s.hi, s.lo);
    s.lo = __dadd_rn(s.lo, t.lo);
    return dd_quick(s.hi, s.lo);
}
__device__ inline DD dd_mul(DD a, DD b) {
    double p = __dmul_rn(a.hi, b.hi);
    double e = __fma_rn(a.hi, b.hi, -p);
    e = __dadd_rn(e, __dadd_rn(__dmul_rn(a.hi, b.lo), __dmul_rn(a.lo, b.hi)));
    return dd_quick(p, e);
}

struct SinCoef { double hi[21]; double lo[21]; };

__device__ inline double sin_cr(double x, const SinCoef &c) {
    DD xd{x, 0.0};
    DD x2 = dd_mul(xd, xd);
    DD acc{c.hi[20], c.lo[20]};
#pragma unroll 1
    for (int k = 19; k >= 0; --k) acc = dd_add(dd_mul(acc, x2), DD{c.hi[k], c.lo[k]});
    acc = dd_mul(acc, xd);
    return __dadd_rn(acc.hi, acc.lo);
}

/* ---- degree_per_meter_longitude (util/util.h:59-66) ---------------------- */
__device__ inline double dpm_arg(double lat) {
    double absla = fabs(lat);
    if (absla == 90.0) absla = 89.0;
    return __ddiv_rn(__dmul_rn(__dsub_rn(90.0, absla), kPI), 180.0);
}
__device__ inline double dpm_from_sin(double s) {
    return __ddiv_rn(360.0, __dmul_rn(__dmul_rn(s, 40076.0), 1000.0));
}
/* fast: CUDA sin (a few ulp from the host's) */
__device__ inline double dpm_lon_fast(double lat) { return dpm_from_sin(sin(dpm_arg(lat))); }

/* the three values the host's degree_per_meter_longitude can take when its
 * sin is within one ulp of the correctly rounded value */
__device__ inline void dpm_lon_candidates(double lat, const SinCoef &c, double out[3]) {
    double s = sin_cr(dpm_arg(lat), c);
    out[0] = dpm_from_sin(s);
    out[1] = dpm_from_sin(__longlong_as_double(__double_as_longlong(s) - 1));
    out[2] = dpm_from_sin(__longlong_as_double(__double_as_longlong(s) + 1));
}

/* ---- the reference's distance tests, exact ------------------------------- */
/* Point::distance(p, true) (geometry/geometry.h:40-48) with a given L = dpm_lon(y1) */
__device__ inline double point_dist(double x1, double y1, double x2, double y2, double L, double dpm_lat) {
    double dx = __dsub_rn(x1, x2);
    double dy = __dsub_rn(y1, y2);
    dy = __ddiv_rn(dy, dpm_lat);
    dx = __ddiv_rn(dx, L);
    return __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

/* box::distance(p, true) (geometry/geometry.h:174-185); L = dpm_lon(p.y) */
__device__ inline double box_dist(double lx, double ly, double hx, double hy, double px, double py, double L,
                                  double dpm_lat) {
    if (px >= lx && px <= hx && py >= ly && py <= hy) return 0.0;
    double ax = __dsub_rn(fabs(__dsub_rn(px, __dmul_rn(__dadd_rn(lx, hx), 0.5))), __dmul_rn(__dsub_rn(hx, lx), 0.5));
    double ay = __dsub_rn(fabs(__dsub_rn(py, __dmul_rn(__dadd_rn(ly, hy), 0.5))), __dmul_rn(__dsub_rn(hy, ly), 0.5));
    double dx = ax < 0.0 ? 0.0 : ax;
    double dy = ay < 0.0 ? 0.0 : ay;
    dy = __ddiv_rn(dy, dpm_lat);
    dx = __ddiv_rn(dx, L);
    return __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

/* decision `value(L) <= r` where value is one of the two distances above.
 * With the fast L the decision is final unless the value lies within a
 * relative band of r that covers every L the host libm could produce; inside
 * the band it is re-taken with the three candidate L values.  If those
 * disagree the correctly rounded one decides and *ambiguous is incremented. */
struct ExactCtx {
    double r;
    double dpm_lat;
    double band;          /* absolute band around r */
    const SinCoef *coef;
    unsigned int *ambiguous;
    unsigned int *rechecks;
};

__device__ inline bool point_le_exact(double x1, double y1, double x2, double y2, double Lfast, const ExactCtx &e) {
    double d = point_dist(x1, y1, x2, y2, Lfast, e.dpm_lat);
    if (fabs(d - e.r) > e.band) return d <= e.r;
    double L[3];
    dpm_lon_candidates(y1, *e.coef, L);
    bool r0 = point_dist(x1, y1, x2, y2, L[0], e.dpm_lat) <= e.r;
    bool r1 = point_dist(x1, y1, x2, y2, L[1], e.dpm_lat) <= e.r;
    bool r2 = point_dist(x1, y1, x2, y2, L[2], e.dpm_lat) <= e.r;
    if (e.rechecks) atomicAdd(e.rechecks, 1u);
    if ((r0 != r1 || r0 != r2) && e.ambiguous) atomicAdd(e.ambiguous, 1u);
    return r0;
}

__device__ inline bool box_le_exact(double lx, double ly, double hx, double hy, double px, double py, double Lfast,
                                    const ExactCtx &e) {
    double d = box_dist(lx, ly, hx, hy, px, py, Lfast, e.dpm_lat);
    if (fabs(d - e.r) > e.band) return d <= e.r;
    double L[3];
    dpm_lon_candidates(py, *e.coef, L);
    bool r0 = box_dist(lx, ly, hx, hy, px, py, L[0], e.dpm_lat) <= e.r;
    bool r1 = box_dist(lx, ly, hx, hy, px, py, L[1], e.dpm_lat) <= e.r;
    bool r2 = box_dist(lx, ly, hx, hy, px, py, L[2], e.dpm_lat) <= e.r;
    if (e.rechecks) atomicAdd(e.rechecks, 1u);
    if ((r0 != r1 || r0 != r2) && e.ambiguous) atomicAdd(e.ambiguous, 1u);
    return r0;
}

/* ---- fixed-point frame for screening tests ----------------------------------
 * Every coordinate is also held as a 64-bit integer X = rn((x - ox) * S) with
 * S = 2^k (k chosen so the map spans about 2^40 units), so differences of
 * coordinates are exact integers, each within 1 + 2^-12 units of the exact
 * scaled difference.  A screening test converts the differences to FP32,
 * scales them to metres with cx = 1/(L S) (L = degree_per_meter_longitude of
 * the first point) and cy = 1/(dpm_lat S), and compares q = mx^2 + my^2 with
 * r^2.  With u = 2^-24: cx is within 9u of exact (the FP64 angle rounded
 * once, the rounded degree constant, sinf's 2 ulp and two products), so
 * near the threshold
 *   |q - d^2| <= 2 r (cx + cy) (1 + 2^-12) + 26 u r^2
 * (integer rounding, then 23u from mx^2, 7u from my^2, 1u from the sum and
 * the FP32 r^2 and band arithmetic).  The guard band is about twice that:
 * 4 r (cx + cy) + 64 u r^2.  Outside the band the screening decision equals
 * the reference's FP64 decision (whose own rounding is near 2^-50 relative);
 * inside it the exact FP64 test decides.
 * A coordinate farther than 2^60 units from the origin is clamped; the object
 * then carries cx = NaN, which sends every test it takes part in to the exact
 * path. */
struct Frame {
    double ox, oy;       /* map low corner */
    double S;            /* units per degree, 2^k */
    float kdeg;          /* fl32(kPI / 180) */
    float kc;            /* fl32(40076000 / (360 S)): cx = sin(angle) * kc */
    float cy;            /* metres per unit along y: 1/(dpm_lat S) */
    float r2;            /* r^2 */
    float band0;         /* 64 u r^2 */
    float band1;         /* 4 r */
};

constexpr double kFxLimit = 1152921504606846976.0; /* 2^60 */

/* a node box in fixed point: low x, low y, high x, high y */
struct __align__(32) IBox {
    long long x, y, z, w;
};

__host__ __device__ inline long long fx_coord(double v, double o, double S, bool *clamped) {
    double t = (v - o) * S; /* S is a power of two: the product is exact */
    bool c = false;
    if (!(t < kFxLimit)) { t = kFxLimit; c = true; }
    if (t < -kFxLimit) { t = -kFxLimit; c = true; }
    if (clamped) *clamped = *clamped || c;
#if defined(__CUDA_ARCH__)
    return __double2ll_rn(t);
#else
    return llrint(t);
#endif
}

/* metres per unit along x at latitude lat, FP32 (within 9u of exact) */
__device__ inline float c_of_lat(double lat, const Frame &f) {
    double a = fabs(lat);
    if (a == 90.0) a = 89.0;
    const float t = (float)__dsub_rn(90.0, a);
    return sinf(t * f.kdeg) * f.kc;
}

/* the per-first-point screening limits */
struct Screen {
    float cx, lo, hi;
};
__device__ inline Screen make_screen(float cx, const Frame &f) {
    const float band = f.band0 + f.band1 * (cx + f.cy);
    Screen s;
    s.cx = cx;
    s.lo = f.r2 - band;
    s.hi = f.r2 + band;
    return s;
}

/* integer -> FP32 on the FP32 pipe (I2F issues on the narrow FP64 pipe of
 * sm_103a): for |v| < 2^22 the bits 0x4B400000 + v are the float
 * 1.5*2^23 + v exactly, so one subtraction recovers v */
__device__ inline float small_to_f(int v) { return __fsub_rn(__int_as_float(0x4B400000 + v), 12582912.0f); }

/* correctly rounded FP32 value of d for |d| < 2^44; NaN beyond (2^13
 * map widths apart), which sends the test to the exact path */
__device__ inline float fx_to_f(long long d) {
    /* d = hi 2^22 + lo with lo in [0, 2^22): one rounding in the fma; for
     * |d| < 2^22, hi is 0 or -1 and the fma is exact */
    const long long w = 1ll << 44;
    const int hi = (int)(d >> 22), lo = (int)(d & 0x3FFFFF);
    const float f = __fmaf_rn(small_to_f(hi), 4194304.0f, small_to_f(lo));
    return (d > -w && d < w) ? f : __int_as_float(0x7fc00000);
}

/* 1 within reach, 0 beyond, -1 inside the guard band (or a NaN scale);
 * dx, dy in units */
__device__ inline int fx_screen(long long dx, long long dy, const Screen &s, float cy) {
    const float mx = fx_to_f(dx) * s.cx, my = fx_to_f(dy) * cy;
    const float q = mx * mx + my * my;
    if (q < s.lo) return 1;
    if (q > s.hi) return 0;
    return -1;
}

__host__ __device__ inline IBox fx_box(double lx, double ly, double hx, double hy, const Frame &f) {
    IBox b;
    b.x = fx_coord(lx, f.ox, f.S, nullptr);
    b.y = fx_coord(ly, f.oy, f.S, nullptr);
    b.z = fx_coord(hx, f.ox, f.S, nullptr);
    b.w = fx_coord(hy, f.oy, f.S, nullptr);
    return b;
}

/* box distance screening: the gap from the point to the box along each axis */
__device__ inline int fx_box_screen(const IBox &b, long long px, long long py, const Screen &s, float cy) {
    /* the gaps are taken after the conversion: rounding is monotonic, so the
     * FP32 maximum is the rounded integer maximum (and needs no 64-bit max) */
    const float x1 = fx_to_f(b.x - px), x2 = fx_to_f(px - b.z);
    const float y1 = fx_to_f(b.y - py), y2 = fx_to_f(py - b.w);
    if (!(x1 == x1 && x2 == x2 && y1 == y1 && y2 == y2)) return -1; /* beyond fx_to_f's range */
    const float gx = fmaxf(fmaxf(x1, x2), 0.0f), gy = fmaxf(fmaxf(y1, y2), 0.0f);
    const float mx = gx * s.cx, my = gy * cy;
    const float q = mx * mx + my * my;
    if (q < s.lo) return 1;
    if (q > s.hi) return 0;
    return -1;
}

/* box::width(true) > two_r (geometry/geometry.h:166-172), exact */
__device__ inline bool width_gt_exact(double lx, double hx, double ly, double two_r, const ExactCtx &e) {
    double w = __ddiv_rn(__dsub_rn(hx, lx), dpm_lon_fast(ly));
    /* same relative slack as the distance band */
    if (fabs(w - two_r) > two_r * (e.band / e.r)) return w > two_r;
    double L[3];
    dpm_lon_candidates(ly, *e.coef, L);
    bool r0 = __ddiv_rn(__dsub_rn(hx, lx), L[0]) > two_r;
    bool r1 = __ddiv_rn(__dsub_rn(hx, lx), L[1]) > two_r;
    bool r2 = __ddiv_rn(__dsub_rn(hx, lx), L[2]) > two_r;
    if ((r0 != r1 || r0 != r2) && e.ambiguous) atomicAdd(e.ambiguous, 1u);
    return r0;
}

/* ---- insertion priority of a contact event --------------------------------
 * The reference inserts into its bucket table in the order of its check list
 * (tracing/refinement.cpp:19-30): first the N inside checks in object order,
 * then the appended cross-leaf checks in object order and, per object, in
 * lookup_rec's depth-first order; within a check, leaf members in stored
 * order.  The priority packs (cross, check object, check ordinal, member
 * rank) so that smaller means earlier. */
__device__ inline uint64_t prio_pack(uint32_t cross, uint32_t pid, uint32_t ordinal, uint32_t rank) {
    return ((uint64_t)cross << 63) | ((uint64_t)pid << 36) | ((uint64_t)(ordinal & 0xFFFFFu) << 16) | (rank & 0xFFFFu);
}

/* order-preserving float for atomicMin/atomicMax on the box */
__device__ inline void mbr_extend(uint32_t *m, float x1, float y1, float x2, float y2, uint32_t cur[4]) {
    uint32_t lx = min(fenc(x1), fenc(x2)), hx = max(fenc(x1), fenc(x2));
    uint32_t ly = min(fenc(y1), fenc(y2)), hy = max(fenc(y1), fenc(y2));
    if (lx < cur[0]) atomicMin(&m[0], lx);
    if (ly < cur[1]) atomicMin(&m[1], ly);
    if (hx > cur[2]) atomicMax(&m[2], hx);
    if (hy > cur[3]) atomicMax(&m[3], hy);
}

} // namespace glint

#endif
