/*
 * TEST INFRASTRUCTURE ONLY — CPU oracle for diffvg_gb300's render path.
 *
 * A plain-C restatement of the reference algorithm (BachiLi/diffvg) over the
 * packed scene layout of include/diffvg_gb300.h.  Each function cites the
 * reference file:line it restates.  Floating-point expressions keep the
 * reference's evaluation order and precision (fp32 where it computes in
 * float, fp64 where it promotes to double), because sample classification
 * (inside / outside, within stroke / not) has to agree with the reference to
 * the last bit for images to match at 1e-4.  Build with -ffp-contract=off.
 *
 * What differs from the reference, on purpose:
 *  - Bounding-volume hierarchies are replaced by a per-16x16-tile candidate
 *    list plus the reference's own leaf-level box tests.  The reference sorts
 *    fragments by group id (diffvg.cpp:605-615) and sums integer winding
 *    numbers, so the traversal order does not change results; the leaf tests
 *    are kept because they do (e.g. an open path only counts crossings inside
 *    its bounding box).  Per-path segment order follows the reference's BVH
 *    depth-first leaf order (scene.cpp:602-620, 439-494) where results can
 *    depend on it (closest-point ties, the early return of
 *    use_distance_approx quadratics).
 *  - The stroke quintic's isolator interval list reads an uninitialised slot
 *    when -B/5 falls outside [0,1] (within_distance.h:223-226,
 *    compute_distance.h:198-201).  Here that slot holds -1, i.e. it is
 *    skipped, which is what the reference computes when the stale value is
 *    negative, >= 1 or 0.
 *  - Capacity overflows and unsupported inputs return an error status
 *    instead of failing an assert.
 *  - Per-pixel sums (weight image, filtered colour) are gathered per pixel
 *    instead of scattered with atomics: same terms, different summation order.
 *
 * Parity is pinned against the compiled reference CPU build by the fixtures
 * under tests/golden/ (see tests/golden/make_golden.py).
 */
#define _GNU_SOURCE
#include "dvg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Work counts (compiled in with -DDVG_COUNT_OPS only; oracle/count_work.py)  */
/* ------------------------------------------------------------------------ */
/* The arithmetic of the reference algorithm as restated here, per phase of
 * a call (weight image, sample colours or interior adjoint, filtered
 * resolve, boundary pass): fp32 add / sub / mul / div, fp64 add / sub / mul
 * / div, and calls of sqrt and the transcendental functions (the reference's
 * own precision decides fp32 or fp64).  Comparisons, bounding-box culls,
 * index arithmetic and the traversal are not counted: the count is that of
 * the formulas a sample evaluates once culling is exact.  Root iterations
 * are counted as executed.  The counts are made by hand per formula in the
 * OPS(...) annotations below. */
#ifdef DVG_COUNT_OPS
#include <stdatomic.h>
enum { PH_WEIGHT, PH_RENDER, PH_RESOLVE, PH_EDGE, PH_COUNT };
static __thread int g_phase;
static __thread uint64_t g_ops[PH_COUNT][3];
static _Atomic uint64_t g_ops_total[PH_COUNT][3];
#define OPS(f32, f64, tr) (g_ops[g_phase][0] += (f32), g_ops[g_phase][1] += (f64), g_ops[g_phase][2] += (tr))
/* a task chunk starts from zero: what the scene set-up counted is dropped */
#define PHASE(p) (g_phase = (p), memset(g_ops, 0, sizeof g_ops))
static void ops_flush(void) {
  for (int p = 0; p < PH_COUNT; p++)
    for (int k = 0; k < 3; k++) {
      atomic_fetch_add(&g_ops_total[p][k], g_ops[p][k]);
      g_ops[p][k] = 0;
    }
}
/* phase-major [weight, render, resolve, edge] x [fp32, fp64, transcendental] */
void dvg_oracle_ops(uint64_t out[12], int reset) {
  for (int p = 0; p < PH_COUNT; p++)
    for (int k = 0; k < 3; k++) {
      out[3 * p + k] = atomic_load(&g_ops_total[p][k]);
      if (reset) atomic_store(&g_ops_total[p][k], 0);
    }
}
#else
#define OPS(f32, f64, tr) ((void)0)
#define PHASE(p) ((void)0)
#define ops_flush() ((void)0)
#endif

/* ------------------------------------------------------------------------ */
/* small vector / box / matrix helpers (vector.h, aabb.h, matrix.h)          */
/* ------------------------------------------------------------------------ */
typedef struct { float x, y; } v2;
typedef struct { float x, y, z, w; } v4;
typedef struct { v2 lo, hi; } box2;

static inline v2 V2(float x, float y) { v2 r; r.x = x; r.y = y; return r; }
static inline v4 V4(float x, float y, float z, float w) { v4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
static inline v2 add2(v2 a, v2 b) { return V2(a.x + b.x, a.y + b.y); }
static inline v2 sub2(v2 a, v2 b) { return V2(a.x - b.x, a.y - b.y); }
static inline v2 mul2(v2 a, v2 b) { return V2(a.x * b.x, a.y * b.y); }
static inline v2 scl2(float s, v2 a) { return V2(s * a.x, s * a.y); }
static inline v2 div2s(v2 a, float s) { return V2(a.x / s, a.y / s); }
static inline v2 neg2(v2 a) { return V2(-a.x, -a.y); }
static inline float sum2(v2 a) { return a.x + a.y; }
static inline float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline float lensq2(v2 a) { return a.x * a.x + a.y * a.y; }
static inline float len2(v2 a) { return sqrtf(lensq2(a)); }
/* distance(v0, v1) = length(v1 - v0)  (vector.h:534-553) */
static inline float dist2(v2 a, v2 b) { return len2(sub2(b, a)); }
static inline float distsq2(v2 a, v2 b) { return lensq2(sub2(b, a)); }
static inline v2 normalize2(v2 a) { float l = len2(a); return V2(a.x / l, a.y / l); }
static inline v4 add4(v4 a, v4 b) { return V4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline v4 sub4(v4 a, v4 b) { return V4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline v4 scl4(float s, v4 a) { return V4(s * a.x, s * a.y, s * a.z, s * a.w); }
static inline float dot4(v4 a, v4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
/* reference min / max (diffvg.h:78-88): NaN-propagation follows a<b?a:b */
static inline float rmin(float a, float b) { return a < b ? a : b; }
static inline float rmax(float a, float b) { return a > b ? a : b; }
static inline float sq(float x) { return x * x; }
/* The reference's unqualified cos / sin calls on float arguments bind to the
 * double-precision libm functions (the CPU build imports cos / sin / sincos),
 * so the argument is widened and the result stays double until stored. */
static inline double dcos(float x) { return cos((double)x); }
static inline double dsin(float x) { return sin((double)x); }

static inline box2 box_empty(void) { box2 b; b.lo = V2(INFINITY, INFINITY); b.hi = V2(-INFINITY, -INFINITY); return b; }
/* merge(box, p) (aabb.h:15-20) */
static inline box2 box_add(box2 b, v2 p) {
  box2 r;
  r.lo = V2(rmin(p.x, b.lo.x), rmin(p.y, b.lo.y));
  r.hi = V2(rmax(p.x, b.hi.x), rmax(p.y, b.hi.y));
  return r;
}
/* merge(box0, box1) (aabb.h:22-27) */
static inline box2 box_union(box2 a, box2 b) {
  box2 r;
  r.lo = V2(rmin(a.lo.x, b.lo.x), rmin(a.lo.y, b.lo.y));
  r.hi = V2(rmax(a.hi.x, b.hi.x), rmax(a.hi.y, b.hi.y));
  return r;
}
/* inside(box, p) (aabb.h:29-33) */
static inline int box_in(box2 b, v2 p) { return p.x >= b.lo.x && p.x <= b.hi.x && p.y >= b.lo.y && p.y <= b.hi.y; }
/* inside(box, p, radius) == within_distance(box, p, r) (aabb.h:35-40, 62-66) */
static inline int box_in_r(box2 b, v2 p, float r) {
  return p.x >= b.lo.x - r && p.x <= b.hi.x + r && p.y >= b.lo.y - r && p.y <= b.hi.y + r;
}
/* intersect(box, pt): the winding-ray test (winding_number.h:33-42) */
static inline int box_ray(box2 b, v2 p) {
  if (p.y < b.lo.y || p.y > b.hi.y) return 0;
  if (p.x > b.hi.x) return 0;
  return 1;
}

/* xform_pt (matrix.h:504-511); m row-major */
static inline v2 xform_pt(const float *m, v2 p) {
  float t0 = m[0] * p.x + m[1] * p.y + m[2];
  float t1 = m[3] * p.x + m[4] * p.y + m[5];
  float t2 = m[6] * p.x + m[7] * p.y + m[8];
  return V2(t0 / t2, t1 / t2);
}
/* d_xform_pt (matrix.h:513-538): accumulates into d_m[9] and *d_pt */
static void d_xform_pt(const float *m, v2 pt, v2 d_out, float *d_m, v2 *d_pt) {
  float t0 = m[0] * pt.x + m[1] * pt.y + m[2];
  float t1 = m[3] * pt.x + m[4] * pt.y + m[5];
  float t2 = m[6] * pt.x + m[7] * pt.y + m[8];
  v2 out = V2(t0 / t2, t1 / t2);
  float dt0 = d_out.x / t2, dt1 = d_out.y / t2;
  float dt2 = -(d_out.x * out.x + d_out.y * out.y) / t2;
  d_m[0] += dt0 * pt.x; d_m[1] += dt0 * pt.y; d_m[2] += dt0;
  d_m[3] += dt1 * pt.x; d_m[4] += dt1 * pt.y; d_m[5] += dt1;
  d_m[6] += dt2 * pt.x; d_m[7] += dt2 * pt.y; d_m[8] += dt2;
  d_pt->x += dt0 * m[0] + dt1 * m[3] + dt2 * m[6];
  d_pt->y += dt0 * m[1] + dt1 * m[4] + dt2 * m[7];
}
/* xform_normal (matrix.h:540-544) */
static inline v2 xform_normal(const float *m_inv, v2 n) {
  return normalize2(V2(m_inv[0] * n.x + m_inv[3] * n.y, m_inv[1] * n.x + m_inv[4] * n.y));
}
/* inverse (matrix.h:209-229) */
static void inverse3(const float *m, float *r) {
#define M(i, j) m[3 * (i) + (j)]
  float det = M(0, 0) * (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2)) -
              M(0, 1) * (M(1, 0) * M(2, 2) - M(1, 2) * M(2, 0)) +
              M(0, 2) * (M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0));
  float invdet = 1 / det;
  r[0] = (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2)) * invdet;
  r[1] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) * invdet;
  r[2] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) * invdet;
  r[3] = (M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2)) * invdet;
  r[4] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) * invdet;
  r[5] = (M(1, 0) * M(0, 2) - M(0, 0) * M(1, 2)) * invdet;
  r[6] = (M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1)) * invdet;
  r[7] = (M(2, 0) * M(0, 1) - M(0, 0) * M(2, 1)) * invdet;
  r[8] = (M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1)) * invdet;
#undef M
}

/* ------------------------------------------------------------------------ */
/* pcg32 (pcg.h:11-40)                                                       */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t state, inc; } pcg32;
static inline uint32_t pcg_next(pcg32 *r) {
  uint64_t old = r->state;
  r->state = old * 6364136223846793005ULL + (r->inc | 1);
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((-rot) & 31));
}
static inline float pcg_float(pcg32 *r) {
  union { uint32_t u; float f; } x;
  x.u = (pcg_next(r) >> 9) | 0x3f800000u;
  return x.f - 1.0f;
}
static inline pcg32 pcg_init(int32_t idx, uint64_t seed) {
  pcg32 s;
  s.state = 0U;
  s.inc = (((uint64_t)(int64_t)idx + 1) << 1u) | 1u;
  pcg_next(&s);
  s.state += (0x853c49e6748fea9bULL + seed);
  pcg_next(&s);
  return s;
}

/* ------------------------------------------------------------------------ */
/* root solvers (solve.h:5-59)                                               */
/* ------------------------------------------------------------------------ */
static int solve_quadratic_f(float a, float b, float c, float *t0, float *t1) {
  float discrim = b * b - 4 * a * c;
  OPS(4, 0, 0);
  if (discrim < 0) return 0;
  OPS(4, 0, 1);
  float root = sqrtf(discrim);
  float q = (b < 0) ? -0.5f * (b - root) : -0.5f * (b + root);
  *t0 = q / a;
  *t1 = c / q;
  if (*t0 > *t1) { float tmp = *t0; *t0 = *t1; *t1 = tmp; }
  return 1;
}
static int solve_quadratic_d(double a, double b, double c, double *t0, double *t1) {
  double discrim = b * b - 4 * a * c;
  OPS(0, 4, 0);
  if (discrim < 0) return 0;
  OPS(0, 4, 1);
  double root = sqrt(discrim);
  double q = (b < 0) ? -0.5f * (b - root) : -0.5f * (b + root);
  *t0 = q / a;
  *t1 = c / q;
  if (*t0 > *t1) { double tmp = *t0; *t0 = *t1; *t1 = tmp; }
  return 1;
}
static int solve_cubic_d(double a, double b, double c, double d, double t[3]) {
  if (fabs(a) < 1e-6f) {
    return solve_quadratic_d(b, c, d, &t[0], &t[1]) ? 2 : 0;
  }
  b /= a; c /= a; d /= a;
  double Q = (b * b - 3 * c) / 9.f;
  double R = (2 * b * b * b - 9 * b * c + 27 * d) / 54.f;
  OPS(0, 19, 0);
  if (R * R < Q * Q * Q) {
    OPS(0, 21, 8);
    double theta = acos(R / sqrt(Q * Q * Q));
    t[0] = -2.f * sqrt(Q) * cos(theta / 3.f) - b / 3.f;
    t[1] = -2.f * sqrt(Q) * cos((theta + 2.f * (double)M_PI) / 3.f) - b / 3.f;
    t[2] = -2.f * sqrt(Q) * cos((theta - 2.f * (double)M_PI) / 3.f) - b / 3.f;
    return 3;
  } else {
    OPS(0, 10, 2);
    double A = R > 0 ? -pow(R + sqrt(R * R - Q * Q * Q), (double)(1. / 3.))
                     : pow(-R + sqrt(R * R - Q * Q * Q), (double)(1. / 3.));
    double B = fabs(A) > 1e-6f ? Q / A : 0.0;
    t[0] = (A + B) - b / 3.0;
    return 1;
  }
}
/* solve_cubic<float>: in the reference CPU build the unqualified sqrt / acos
 * / cos / pow calls inside the template bind to the double-precision libm
 * functions (the built module imports acos, cos, pow and no acosf / cosf /
 * powf), so float arguments are promoted and intermediate results are double
 * until they are stored back into a float. */
static int solve_cubic_f(float a, float b, float c, float d, float t[3]) {
  if (fabs(a) < 1e-6f) {
    return solve_quadratic_f(b, c, d, &t[0], &t[1]) ? 2 : 0;
  }
  b /= a; c /= a; d /= a;
  float Q = (b * b - 3 * c) / 9.f;
  float R = (2 * b * b * b - 9 * b * c + 27 * d) / 54.f;
  OPS(19, 0, 0);
  if (R * R < Q * Q * Q) {
    OPS(6, 15, 8);
    float theta = (float)acos((double)R / sqrt((double)(Q * Q * Q)));
    t[0] = (float)(-2.f * sqrt((double)Q) * cos((double)(theta / 3.f)) - (double)(b / 3.f));
    t[1] = (float)(-2.f * sqrt((double)Q) * cos((double)((theta + 2.f * (float)M_PI) / 3.f)) - (double)(b / 3.f));
    t[2] = (float)(-2.f * sqrt((double)Q) * cos((double)((theta - 2.f * (float)M_PI) / 3.f)) - (double)(b / 3.f));
    return 3;
  } else {
    OPS(4, 6, 2);
    double third = (double)(float)(1. / 3.);
    float A = R > 0 ? (float)(-pow((double)R + sqrt((double)(R * R - Q * Q * Q)), third))
                    : (float)pow((double)(-R) + sqrt((double)(R * R - Q * Q * Q)), third);
    float B = fabs(A) > 1e-6f ? Q / A : 0.f;
    t[0] = (A + B) - b / 3.f;
    return 1;
  }
}

/* ------------------------------------------------------------------------ */
/* pixel filters (filter.h:22-106)                                           */
/* ------------------------------------------------------------------------ */
/* DVG_GAUSSIAN is not in the reference: the definition of this project's
 * kernels (separable Gaussian, standard deviation r / 2, shifted to 0 at the
 * edge of the support), checked by finite differences only. */
static float gauss_1d(float x, float r) { return expf(-2.f * sq(x) / sq(r)) - expf(-2.f); }
static float filter_weight(int type, float r, float dx, float dy) {
  if (fabsf(dx) > r || fabsf(dy) > r) return 0;
  OPS(type == DVG_BOX ? 3 : type == DVG_TENT ? 6 : type == DVG_PARABOLIC ? 10 : type == DVG_HANN ? 16 : 12, 0,
      type == DVG_HANN || type == DVG_GAUSSIAN ? 2 : 0);
  if (type == DVG_GAUSSIAN) return r > 0.f ? gauss_1d(dx, r) * gauss_1d(dy, r) : 0.f;
  if (type == DVG_BOX) return 1.f / sq(2 * r);
  if (type == DVG_TENT) return (r - fabsf(dx)) * (r - fabsf(dy)) / sq(sq(r));
  if (type == DVG_PARABOLIC)
    return (4.f / 3.f) * (1 - sq(dx / r)) * (4.f / 3.f) * (1 - sq(dy / r));
  {
    float ndx = (dx / (2 * r)) + 0.5f, ndy = (dy / (2 * r)) + 0.5f;
    return 0.5f * (1.f - cosf((float)(2 * M_PI) * ndx)) * 0.5f * (1.f - cosf((float)(2 * M_PI) * ndy)) / sq(r);
  }
}
static float d_filter_weight(int type, float r, float dx, float dy, float d_ret) {
  OPS(type == DVG_BOX ? 7 : type == DVG_TENT ? 14 : type == DVG_PARABOLIC ? 9 : 40, 0,
      type == DVG_HANN || type == DVG_GAUSSIAN ? 4 : (type == DVG_TENT ? 1 : 0));
  if (type == DVG_GAUSSIAN) {
    if (!(r > 0.f) || fabsf(dx) > r || fabsf(dy) > r) return 0.f;
    float r3 = r * r * r;
    float dgx = expf(-2.f * sq(dx) / sq(r)) * 4.f * sq(dx) / r3, dgy = expf(-2.f * sq(dy) / sq(r)) * 4.f * sq(dy) / r3;
    return d_ret * (dgx * gauss_1d(dy, r) + gauss_1d(dx, r) * dgy);
  }
  if (type == DVG_BOX) {
    return d_ret * (-2) * 2 * r / ((2 * r) * (2 * r) * (2 * r));
  } else if (type == DVG_TENT) {
    float fx = r - fabsf(dx), fy = r - fabsf(dy);
    float norm = 1 / sq(r);
    float d_fx = d_ret * fy * norm, d_fy = d_ret * fx * norm, d_norm = d_ret * fx * fy;
    return d_fx + d_fy + (-4) * d_norm / (float)pow(r, 5);
  } else if (type == DVG_PARABOLIC) {
    float r3 = r * r * r;
    return -(2 * sq(dx) + 2 * sq(dy)) / r3;
  } else {
    float ndx = (dx / (2 * r)) + 0.5f, ndy = (dy / (2 * r)) + 0.5f;
    float fx = 0.5f * (1.f - cosf((float)(2 * M_PI) * ndx));
    float fy = 0.5f * (1.f - cosf((float)(2 * M_PI) * ndy));
    float norm = 1 / sq(r);
    float d_fx = d_ret * fy * norm, d_fy = d_ret * fx * norm, d_norm = d_ret * fx * fy;
    float d_ndx = d_fx * 0.5f * sinf((float)(2 * M_PI) * ndx) * (float)(2 * M_PI);
    float d_ndy = d_fy * 0.5f * sinf((float)(2 * M_PI) * ndy) * (float)(2 * M_PI);
    return d_ndx * (-2 * dx / sq(2 * r)) + d_ndy * (-2 * dy / sq(2 * r)) + (-2) * d_norm / (r * r * r);
  }
}

/* ------------------------------------------------------------------------ */
/* scene                                                                     */
/* ------------------------------------------------------------------------ */
#define TILE 16
#define MAX_FRAGMENTS 256          /* diffvg.cpp:542 */
#define MAX_PREFILTER_FRAGMENTS 64 /* diffvg.cpp:847 */

typedef struct {
  const DvgSceneDesc *d;
  const float *P;
  int W, H;                /* canvas */
  /* per group */
  float *c2s;              /* [G*9] */
  box2 *g_local_box;       /* union of the group's shape boxes (local space) */
  box2 *g_canvas_box;
  float *g_max_radius;
  /* per shape */
  box2 *s_box;
  float *s_length;
  /* per segment (global index) */
  int *seg_point;          /* first point index of the segment */
  box2 *seg_box;
  float *seg_r;            /* max stroke radius over the segment's points */
  float *seg_pmf, *seg_cdf;
  int *seg_order;          /* per path: BVH depth-first leaf order (local indices) */
  /* edge sampling */
  int num_total;
  float *smp_cdf, *smp_pmf;
  int *smp_shape, *smp_group;
  /* tile candidate lists */
  int tx, ty;
  int *tile_start, *tile_list;
  int *all_groups;
} Scene;

#define SI(S, s, f) ((S)->d->shape_info[(s) * DVG_SHAPE_INFO_STRIDE + (f)])
#define GI(S, g, f) ((S)->d->group_info[(g) * DVG_GROUP_INFO_STRIDE + (f)])

static __thread char *g_err;
static __thread int g_err_len;
static __thread int g_status;
static void fail(int status, const char *fmt, ...) {
  if (g_status != DVG_OK) return;
  g_status = status;
  if (g_err && g_err_len > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, (size_t)g_err_len, fmt, ap);
    va_end(ap);
  }
}
/* worker threads report errors through a shared word */
static _Atomic int g_worker_status;
static void worker_fail(int status) {
  int expected = DVG_OK;
  atomic_compare_exchange_strong(&g_worker_status, &expected, status);
}

static inline v2 path_pt(const Scene *S, int s, int i) {
  const float *p = S->P + SI(S, s, DVG_SHAPE_PARAM_OFF);
  return V2(p[2 * i], p[2 * i + 1]);
}
static inline float stroke_width(const Scene *S, int s) { return S->P[SI(S, s, DVG_SHAPE_STROKE_WIDTH_OFF)]; }

/* eval of a Bezier segment (within_distance.h:63-66, 128-131) */
static inline v2 eval_quad(v2 p0, v2 p1, v2 p2, float t) {
  OPS(15, 0, 0);
  float tt = 1 - t;
  return add2(add2(scl2(tt * tt, p0), scl2(2 * tt * t, p1)), scl2(t * t, p2));
}
static inline v2 eval_cubic(v2 p0, v2 p1, v2 p2, v2 p3, float t) {
  OPS(25, 0, 0);
  float tt = 1 - t;
  return add2(add2(add2(scl2(tt * tt * tt, p0), scl2(3 * tt * tt * t, p1)), scl2(3 * tt * t * t, p2)),
              scl2(t * t * t, p3));
}


/* per-path BVH leaf order: segments sorted by box y-centre, paired bottom-up
 * (scene.cpp:439-494, 602-620), visited depth-first with child1 before child0
 * (winding_number.h:44-172 stack discipline). */
static void path_leaf_order(const box2 *boxes, int n, int *out) {
  int *idx = (int *)malloc(sizeof(int) * (size_t)n);
  float *key = (float *)malloc(sizeof(float) * (size_t)n);
  for (int i = 0; i < n; i++) { idx[i] = i; key[i] = 0.5f * (boxes[i].lo.y + boxes[i].hi.y); }
  /* stable insertion sort by key */
  for (int i = 1; i < n; i++) {
    int v = idx[i]; int j = i;
    while (j > 0 && key[idx[j - 1]] > key[v]) { idx[j] = idx[j - 1]; j--; }
    idx[j] = v;
  }
  if (n == 1) { out[0] = idx[0]; free(idx); free(key); return; }
  int size = 2 * n - 1;
  int *c0 = (int *)malloc(sizeof(int) * (size_t)size), *c1 = (int *)malloc(sizeof(int) * (size_t)size);
  for (int i = 0; i < size; i++) { c0[i] = -1; c1[i] = -1; }
  int prev_beg = 0, prev_end = n;
  int leftover = prev_end % 2 == 0 ? -1 : prev_end - 1;
  while (prev_end - prev_beg >= 1 || leftover != -1) {
    int length = (prev_end - prev_beg) / 2;
    if ((prev_end - prev_beg) % 2 == 1 && leftover != -1 && leftover != prev_end - 1) length += 1;
    for (int i = 0; i < length; i++) {
      int a = prev_beg + 2 * i, b = prev_beg + 2 * i + 1;
      if (b >= prev_end) { b = leftover; leftover = -1; }
      c0[prev_end + i] = a; c1[prev_end + i] = b;
    }
    if (length == 1 && leftover == -1) break;
    prev_beg = prev_end;
    prev_end = prev_beg + length;
    if (length % 2 == 1 && leftover == -1) leftover = prev_end - 1;
  }
  int *stack = (int *)malloc(sizeof(int) * (size_t)(size + 1));
  int sp = 0, k = 0;
  stack[sp++] = size - 1;
  while (sp > 0) {
    int node = stack[--sp];
    if (node < n) { out[k++] = idx[node]; continue; }
    stack[sp++] = c0[node];
    stack[sp++] = c1[node];
  }
  free(stack); free(c0); free(c1); free(idx); free(key);
}

static int scene_init(Scene *S, const DvgSceneDesc *d, const float *P) {
  memset(S, 0, sizeof(*S));
  S->d = d; S->P = P; S->W = d->canvas_width; S->H = d->canvas_height;
  int G = d->num_groups, NS = d->num_shapes, NSEG = d->total_segments;
  S->c2s = (float *)calloc((size_t)(G > 0 ? G : 1) * 9, sizeof(float));
  S->g_local_box = (box2 *)calloc((size_t)(G > 0 ? G : 1), sizeof(box2));
  S->g_canvas_box = (box2 *)calloc((size_t)(G > 0 ? G : 1), sizeof(box2));
  S->g_max_radius = (float *)calloc((size_t)(G > 0 ? G : 1), sizeof(float));
  S->s_box = (box2 *)calloc((size_t)(NS > 0 ? NS : 1), sizeof(box2));
  S->s_length = (float *)calloc((size_t)(NS > 0 ? NS : 1), sizeof(float));
  S->seg_point = (int *)calloc((size_t)(NSEG > 0 ? NSEG : 1), sizeof(int));
  S->seg_box = (box2 *)calloc((size_t)(NSEG > 0 ? NSEG : 1), sizeof(box2));
  S->seg_r = (float *)calloc((size_t)(NSEG > 0 ? NSEG : 1), sizeof(float));
  S->seg_pmf = (float *)calloc((size_t)(NSEG > 0 ? NSEG : 1), sizeof(float));
  S->seg_cdf = (float *)calloc((size_t)(NSEG > 0 ? NSEG : 1), sizeof(float));
  S->seg_order = (int *)calloc((size_t)(NSEG > 0 ? NSEG : 1), sizeof(int));

  for (int g = 0; g < G; g++) inverse3(P + GI(S, g, DVG_GROUP_XFORM_OFF), S->c2s + 9 * g);

  /* shape boxes, segment boxes and radii (scene.cpp:495-625) */
  for (int s = 0; s < NS; s++) {
    int kind = SI(S, s, DVG_SHAPE_KIND);
    const float *p = P + SI(S, s, DVG_SHAPE_PARAM_OFF);
    if (kind == DVG_CIRCLE) {
      float r = p[0]; v2 c = V2(p[1], p[2]);
      S->s_box[s].lo = V2(c.x - r, c.y - r); S->s_box[s].hi = V2(c.x + r, c.y + r);
    } else if (kind == DVG_ELLIPSE) {
      v2 r = V2(p[0], p[1]), c = V2(p[2], p[3]);
      S->s_box[s].lo = sub2(c, r); S->s_box[s].hi = add2(c, r);
    } else if (kind == DVG_RECT) {
      S->s_box[s].lo = V2(p[0], p[1]); S->s_box[s].hi = V2(p[2], p[3]);
    } else if (kind == DVG_PATH) {
      int np = SI(S, s, DVG_SHAPE_NUM_POINTS), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS);
      int so = SI(S, s, DVG_SHAPE_SEG_OFF), th = SI(S, s, DVG_SHAPE_THICKNESS_OFF);
      box2 b = box_empty();
      if (np > 0) { b.lo = path_pt(S, s, 0); b.hi = b.lo; }
      for (int i = 1; i < np; i++) b = box_add(b, path_pt(S, s, i));
      S->s_box[s] = b;
      float r = stroke_width(S, s);
      int pid = 0;
      for (int i = 0; i < nseg; i++) {
        int nc = d->segment_ctrl[so + i];
        S->seg_point[so + i] = pid;
        box2 sb = box_empty();
        float rr = r;
        for (int k = 0; k <= nc + 1; k++) {
          int id = (k == nc + 1) ? (pid + k) % np : pid + k;
          sb = box_add(sb, path_pt(S, s, id));
          if (th >= 0) {
            float rk = P[th + id];
            rr = (k == 0) ? rk : rmax(rr, rk);
          }
        }
        S->seg_box[so + i] = sb;
        S->seg_r[so + i] = rr;
        pid += nc + 1;
      }
      if (nseg > 0) path_leaf_order(S->seg_box + so, nseg, S->seg_order + so);
    }
  }
  /* group boxes and top-level radii (scene.cpp:627-684) */
  for (int g = 0; g < G; g++) {
    int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
    box2 b = box_empty();
    float max_r = 0.f;
    for (int k = 0; k < nsh; k++) {
      int s = d->group_shapes[off + k];
      b = (k == 0) ? S->s_box[s] : box_union(b, S->s_box[s]);
      float r = stroke_width(S, s);
      if (SI(S, s, DVG_SHAPE_KIND) == DVG_PATH && SI(S, s, DVG_SHAPE_THICKNESS_OFF) >= 0 &&
          SI(S, s, DVG_SHAPE_NUM_SEGMENTS) > 0) {
        /* the reference reads node 0 of the path BVH: the leaf with the lowest y-centre */
        int so = SI(S, s, DVG_SHAPE_SEG_OFF), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS);
        int best = 0;
        float bk = 0.5f * (S->seg_box[so].lo.y + S->seg_box[so].hi.y);
        for (int i = 1; i < nseg; i++) {
          float ki = 0.5f * (S->seg_box[so + i].lo.y + S->seg_box[so + i].hi.y);
          if (ki < bk) { bk = ki; best = i; }
        }
        r = S->seg_r[so + best];
      }
      max_r = (k == 0) ? r : (max_r < r ? r : max_r); /* std::max */
    }
    S->g_local_box[g] = b;
    const float *m = P + GI(S, g, DVG_GROUP_XFORM_OFF);
    box2 cb = box_empty();
    cb = box_add(cb, xform_pt(m, V2(b.lo.x, b.lo.y)));
    cb = box_add(cb, xform_pt(m, V2(b.lo.x, b.hi.y)));
    cb = box_add(cb, xform_pt(m, V2(b.hi.x, b.lo.y)));
    cb = box_add(cb, xform_pt(m, V2(b.hi.x, b.hi.y)));
    S->g_canvas_box[g] = cb;
    S->g_max_radius[g] = GI(S, g, DVG_GROUP_STROKE_KIND) == DVG_PAINT_NONE ? 0.f : max_r;
  }

  /* boundary lengths and sampling distributions (scene.cpp:113-333) */
  for (int s = 0; s < NS; s++) {
    int kind = SI(S, s, DVG_SHAPE_KIND);
    const float *p = P + SI(S, s, DVG_SHAPE_PARAM_OFF);
    float L = 0.f;
    if (kind == DVG_CIRCLE) {
      L += (float)(2.f * M_PI) * p[0];
    } else if (kind == DVG_ELLIPSE) {
      float a = p[0], b = p[1];
      L += (float)((float)M_PI * (3 * (a + b) - sqrt((double)((3 * a + b) * (a + 3 * b)))));
    } else if (kind == DVG_RECT) {
      L += 2 * (p[2] - p[0] + p[3] - p[1]);
    } else if (kind == DVG_PATH) {
      int np = SI(S, s, DVG_SHAPE_NUM_POINTS), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
      float len = 0.f;
      for (int i = 0; i < nseg; i++) {
        int nc = d->segment_ctrl[so + i], i0 = S->seg_point[so + i];
        if (nc == 0) {
          len += dist2(path_pt(S, s, (i0 + 1) % np), path_pt(S, s, i0));
        } else if (nc == 1) {
          v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, (i0 + 2) % np);
          v2 v1 = eval_quad(p0, p1, p2, 0.5f);
          len += dist2(v1, p0) + dist2(v1, p2);
        } else {
          v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, i0 + 2), p3 = path_pt(S, s, (i0 + 3) % np);
          v2 v1 = eval_cubic(p0, p1, p2, p3, 1.f / 3.f), v2_ = eval_cubic(p0, p1, p2, p3, 2.f / 3.f);
          len += dist2(v1, p0) + dist2(v1, v2_) + dist2(v2_, p3);
        }
      }
      L += len;
      float inv = 1.f / L;
      for (int i = 0; i < nseg; i++) {
        int nc = d->segment_ctrl[so + i], i0 = S->seg_point[so + i];
        float dd;
        if (nc == 0) {
          dd = dist2(path_pt(S, s, i0), path_pt(S, s, (i0 + 1) % np)) * inv;
        } else if (nc == 1) {
          v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, (i0 + 2) % np);
          v2 v1 = eval_quad(p0, p1, p2, 0.5f);
          dd = (dist2(p0, v1) + dist2(v1, p2)) * inv;
        } else {
          v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, i0 + 2), p3 = path_pt(S, s, (i0 + 3) % np);
          v2 v1 = eval_cubic(p0, p1, p2, p3, 1.f / 3.f), v2_ = eval_cubic(p0, p1, p2, p3, 2.f / 3.f);
          dd = (dist2(v1, p0) + dist2(v1, v2_) + dist2(v2_, p3)) * inv;
        }
        S->seg_pmf[so + i] = dd;
        S->seg_cdf[so + i] = (i == 0) ? dd : dd + S->seg_cdf[so + i - 1];
      }
    }
    S->s_length[s] = L;
  }
  int nt = 0;
  for (int g = 0; g < G; g++) nt += GI(S, g, DVG_GROUP_NUM_SHAPES);
  S->num_total = nt;
  S->smp_cdf = (float *)calloc((size_t)(nt > 0 ? nt : 1), sizeof(float));
  S->smp_pmf = (float *)calloc((size_t)(nt > 0 ? nt : 1), sizeof(float));
  S->smp_shape = (int *)calloc((size_t)(nt > 0 ? nt : 1), sizeof(int));
  S->smp_group = (int *)calloc((size_t)(nt > 0 ? nt : 1), sizeof(int));
  int k = 0;
  for (int g = 0; g < G; g++) {
    int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
    for (int i = 0; i < nsh; i++) {
      int s = d->group_shapes[off + i];
      float len = S->s_length[s];
      S->smp_shape[k] = s;
      S->smp_cdf[k] = (k == 0) ? len : len + S->smp_cdf[k - 1];
      S->smp_pmf[k] = len;
      S->smp_group[k] = g;
      k++;
    }
  }
  if (nt > 0) {
    float norm = S->smp_cdf[nt - 1];
    if (norm <= 0) {
      fail(DVG_ERR_SCENE, "The total length of the shape boundaries in the scene is equal or less than 0. Length = %f", norm);
      return -1;
    }
    if (!isfinite(norm)) {
      fail(DVG_ERR_SCENE, "The total length of the shape boundaries in the scene is not a number. Length = %f", norm);
      return -1;
    }
    for (int i = 0; i < nt; i++) { S->smp_cdf[i] /= norm; S->smp_pmf[i] /= norm; }
  }

  /* per-tile candidate lists, conservative w.r.t. the top-level leaf test */
  S->tx = (S->W + TILE - 1) / TILE; S->ty = (S->H + TILE - 1) / TILE;
  if (S->tx < 1) S->tx = 1;
  if (S->ty < 1) S->ty = 1;
  int NT = S->tx * S->ty;
  int *cnt = (int *)calloc((size_t)NT + 1, sizeof(int));
  int *lo = (int *)malloc(sizeof(int) * 4 * (size_t)(G > 0 ? G : 1));
  for (int g = 0; g < G; g++) {
    box2 b = S->g_canvas_box[g];
    float r = S->g_max_radius[g];
    int x0, x1, y0, y1;
    if (G == 1) { x0 = 0; x1 = S->tx - 1; y0 = 0; y1 = S->ty - 1; }
    else {
      double fx0 = floor(((double)b.lo.x - r - 1.0) / TILE), fx1 = floor(((double)b.hi.x + r + 1.0) / TILE);
      double fy0 = floor(((double)b.lo.y - r - 1.0) / TILE), fy1 = floor(((double)b.hi.y + r + 1.0) / TILE);
      if (!(fx0 <= fx1) || !(fy0 <= fy1)) { x0 = 1; x1 = 0; y0 = 1; y1 = 0; }
      else {
        x0 = fx0 < 0 ? 0 : (fx0 > S->tx - 1 ? S->tx : (int)fx0);
        x1 = fx1 > S->tx - 1 ? S->tx - 1 : (fx1 < 0 ? -1 : (int)fx1);
        y0 = fy0 < 0 ? 0 : (fy0 > S->ty - 1 ? S->ty : (int)fy0);
        y1 = fy1 > S->ty - 1 ? S->ty - 1 : (fy1 < 0 ? -1 : (int)fy1);
      }
    }
    lo[4 * g] = x0; lo[4 * g + 1] = x1; lo[4 * g + 2] = y0; lo[4 * g + 3] = y1;
    for (int y = y0; y <= y1; y++)
      for (int x = x0; x <= x1; x++) cnt[y * S->tx + x]++;
  }
  S->tile_start = (int *)calloc((size_t)NT + 1, sizeof(int));
  for (int t = 0; t < NT; t++) S->tile_start[t + 1] = S->tile_start[t] + cnt[t];
  S->tile_list = (int *)malloc(sizeof(int) * (size_t)(S->tile_start[NT] > 0 ? S->tile_start[NT] : 1));
  memset(cnt, 0, sizeof(int) * (size_t)NT);
  for (int g = 0; g < G; g++) /* ascending group order inside every list */
    for (int y = lo[4 * g + 2]; y <= lo[4 * g + 3]; y++)
      for (int x = lo[4 * g]; x <= lo[4 * g + 1]; x++) {
        int t = y * S->tx + x;
        S->tile_list[S->tile_start[t] + cnt[t]++] = g;
      }
  S->all_groups = (int *)malloc(sizeof(int) * (size_t)(G > 0 ? G : 1));
  for (int g = 0; g < G; g++) S->all_groups[g] = g;
  free(cnt); free(lo);
  return 0;
}

static void scene_free(Scene *S) {
  free(S->c2s); free(S->g_local_box); free(S->g_canvas_box); free(S->g_max_radius);
  free(S->s_box); free(S->s_length); free(S->seg_point); free(S->seg_box); free(S->seg_r);
  free(S->seg_pmf); free(S->seg_cdf); free(S->seg_order);
  free(S->smp_cdf); free(S->smp_pmf); free(S->smp_shape); free(S->smp_group);
  free(S->tile_start); free(S->tile_list); free(S->all_groups);
}

/* candidate groups for a canvas-space point (ascending group id) */
static const int *candidates(const Scene *S, v2 pt, int *n) {
  float fx = floorf(pt.x / TILE), fy = floorf(pt.y / TILE);
  if (fx >= 0 && fy >= 0 && fx < S->tx && fy < S->ty) {
    int t = (int)fy * S->tx + (int)fx;
    *n = S->tile_start[t + 1] - S->tile_start[t];
    return S->tile_list + S->tile_start[t];
  }
  *n = S->d->num_groups;
  return S->all_groups;
}

/* ------------------------------------------------------------------------ */
/* winding numbers (winding_number.h:9-202)                                  */
/* ------------------------------------------------------------------------ */
static int winding_segment(const Scene *S, int s, int seg, v2 pt) {
  int so = SI(S, s, DVG_SHAPE_SEG_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
  int nc = S->d->segment_ctrl[so + seg], i0 = S->seg_point[so + seg];
  int w = 0;
  if (nc == 0) {
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, (i0 + 1) % np);
    if (p1.y != p0.y) {
      float t = (pt.y - p0.y) / (p1.y - p0.y);
      OPS(3, 0, 0);
      if (t >= 0 && t <= 1) {
        OPS(5, 0, 0);
        float tp = p0.x - pt.x + t * (p1.x - p0.x);
        if (tp >= 0) w += (p1.y - p0.y > 0) ? 1 : -1;
      }
    }
  } else if (nc == 1) {
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, (i0 + 2) % np);
    float t[2];
    OPS(7, 0, 0);
    if (solve_quadratic_f(p0.y - 2 * p1.y + p2.y, -2 * p0.y + 2 * p1.y, p0.y - pt.y, &t[0], &t[1])) {
      for (int j = 0; j < 2; j++) {
        if (t[j] >= 0 && t[j] <= 1) {
          OPS(19, 0, 0);
          float tp = (p0.x - 2 * p1.x + p2.x) * t[j] * t[j] + (-2 * p0.x + 2 * p1.x) * t[j] + p0.x - pt.x;
          if (tp >= 0) w += (2 * (p0.y - 2 * p1.y + p2.y) * t[j] + (-2 * p0.y + 2 * p1.y) > 0) ? 1 : -1;
        }
      }
    }
  } else {
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, i0 + 2), p3 = path_pt(S, s, (i0 + 3) % np);
    double t[3];
    OPS(14, 0, 0);
    int n = solve_cubic_d((double)(-p0.y + 3 * p1.y - 3 * p2.y + p3.y), (double)(3 * p0.y - 6 * p1.y + 3 * p2.y),
                          (double)(-3 * p0.y + 3 * p1.y), (double)(p0.y - pt.y), t);
    for (int j = 0; j < n; j++) {
      if (t[j] >= 0 && t[j] <= 1) {
        OPS(27, 18, 0);
        double tp = (-p0.x + 3 * p1.x - 3 * p2.x + p3.x) * t[j] * t[j] * t[j] +
                    (3 * p0.x - 6 * p1.x + 3 * p2.x) * t[j] * t[j] + (-3 * p0.x + 3 * p1.x) * t[j] + p0.x - pt.x;
        if (tp > 0) {
          w += (3 * (-p0.y + 3 * p1.y - 3 * p2.y + p3.y) * t[j] * t[j] + 2 * (3 * p0.y - 6 * p1.y + 3 * p2.y) * t[j] +
                (-3 * p0.y + 3 * p1.y) > 0) ? 1 : -1;
        }
      }
    }
  }
  return w;
}

static int winding_shape(const Scene *S, int s, v2 pt) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  const float *p = S->P + SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    v2 c = V2(p[1], p[2]); float r = p[0];
    return distsq2(c, pt) < r * r ? 1 : 0;
  } else if (kind == DVG_ELLIPSE) {
    v2 r = V2(p[0], p[1]), c = V2(p[2], p[3]);
    return (sq(c.x - pt.x) / sq(r.x) + sq(c.y - pt.y) / sq(r.y) < 1) ? 1 : 0;
  } else if (kind == DVG_RECT) {
    return (pt.x > p[0] && pt.x < p[2] && pt.y > p[1] && pt.y < p[3]) ? 1 : 0;
  } else {
    int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
    int w = 0;
    for (int i = 0; i < nseg; i++) {
      if (nseg > 1 && !box_ray(S->seg_box[so + i], pt)) continue;
      w += winding_segment(S, s, i, pt);
    }
    return w;
  }
}

typedef struct { int group, shape, hit; } EdgeQ;

/* is_inside (diffvg.cpp:33-87) */
static int group_inside(const Scene *S, int g, v2 pt, EdgeQ *eq) {
  v2 lp = xform_pt(S->c2s + 9 * g, pt);
  OPS(14, 0, 0);
  if (!box_in(S->g_local_box[g], lp)) return 0;
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  int eo = GI(S, g, DVG_GROUP_EVEN_ODD);
  int w = 0;
  for (int k = 0; k < nsh; k++) {
    int s = S->d->group_shapes[off + k];
    if (nsh > 1 && !box_in(S->s_box[s], lp)) continue;
    int ws = winding_shape(S, s, lp);
    w += ws;
    if (eq && eq->group == g && eq->shape == s) {
      if ((eo && abs(ws) % 2 == 1) || (!eo && ws != 0)) eq->hit = 1;
    }
  }
  return eo ? (abs(w) % 2 == 1) : (w != 0);
}

/* ------------------------------------------------------------------------ */
/* stroke coverage (within_distance.h:8-446)                                 */
/* ------------------------------------------------------------------------ */
static inline float det2(v2 a, v2 b) { return a.x * b.y - b.x * a.y; }
static inline float clampf_(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
/* quadratic_closest_pt_approx (vector.h:787-817) */
static v2 quad_closest_approx(v2 b0, v2 b1, v2 b2, v2 pt, float *t_out) {
  b0 = sub2(b0, pt); b1 = sub2(b1, pt); b2 = sub2(b2, pt);
  float a = det2(b0, b2), b = 2 * det2(b1, b0), d = 2 * det2(b2, b1);
  float f = b * d - a * a;
  v2 d21 = sub2(b2, b1), d10 = sub2(b1, b0), d20 = sub2(b2, b0);
  v2 gf = scl2(2, add2(add2(scl2(b, d21), scl2(d, d10)), scl2(a, d20)));
  gf = V2(gf.y, -gf.x);
  v2 pp = div2s(scl2(-f, gf), dot2(gf, gf));
  v2 d0p = sub2(b0, pp);
  float ap = det2(d0p, d20), bp = 2 * det2(d10, d0p);
  float t = clampf_((ap + bp) / (2 * a + b + d), 0.f, 1.f);
  float tt = 1 - t;
  if (t_out) *t_out = t;
  return add2(add2(add2(scl2(tt * tt, b0), scl2(2 * tt * t, b1)), scl2(t * t, b2)), pt);
}

/* coefficients of the cubic-segment distance quintic (within_distance.h:150-167) */
typedef struct { double A, B, C, D, E, F; } Quintic;
static Quintic cubic_quintic(v2 p0, v2 p1, v2 p2, v2 p3, v2 pt) {
  v2 a = add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3);
  v2 b = add2(sub2(scl2(3, p0), scl2(6, p1)), scl2(3, p2));
  v2 c = add2(scl2(-3, p0), scl2(3, p1));
  v2 e = sub2(p0, pt);
  Quintic q;
  OPS(66, 5, 0);
  q.A = (double)(3 * sum2(mul2(a, a)));
  q.B = (double)(5 * sum2(mul2(a, b)));
  q.C = (double)(4 * sum2(mul2(a, c)) + 2 * sum2(mul2(b, b)));
  q.D = (double)(3 * (sum2(mul2(b, c)) + sum2(mul2(a, e))));
  q.E = (double)(sum2(mul2(c, c)) + 2 * sum2(mul2(e, b)));
  q.F = (double)(sum2(mul2(e, c)));
  q.B /= q.A; q.C /= q.A; q.D /= q.A; q.E /= q.A; q.F /= q.A;
  return q;
}
static inline double quintic_eval(const Quintic *q, double t) {
  OPS(0, 19, 0);
  return t * t * t * t * t + q->B * t * t * t * t + q->C * t * t * t + q->D * t * t + q->E * t + q->F;
}
static inline double quintic_deriv(const Quintic *q, double t) {
  OPS(0, 17, 0);
  return 5 * t * t * t * t + 4 * q->B * t * t * t + 3 * q->C * t * t + 2 * q->D * t + q->E;
}
/* isolator intervals of the normalised quintic (within_distance.h:181-236);
 * returns the number of entries written to iv[4]. */
static int quintic_intervals(const Quintic *q, float iv[4]) {
  double p1A = (2 / 5.f) * q->C - (4 / 25.f) * q->B * q->B;
  double p1B = (3 / 5.f) * q->D - (3 / 25.f) * q->B * q->C;
  double p1C = (4 / 5.f) * q->E - (2 / 25.f) * q->B * q->D;
  double p1D = q->F - q->B * q->E / 25.f;
  double q_root = -q->B / 5.f;
  double pr[3];
  OPS(0, 17, 0);
  int ns = solve_cubic_d(p1A, p1B, p1C, p1D, pr);
  iv[0] = (q_root >= 0 && q_root <= 1) ? (float)q_root : -1.0f;
  for (int j = 0; j < ns; j++) iv[j + 1] = (float)pr[j];
  int n = 1 + ns;
  for (int j = 1; j < n; j++)
    for (int k = j; k > 0 && iv[k - 1] > iv[k]; k--) { float tmp = iv[k]; iv[k] = iv[k - 1]; iv[k - 1] = tmp; }
  return n;
}
/* safeguarded Newton / bisection inside one bracket (within_distance.h:251-269) */
static float quintic_root(const Quintic *q, float lb, float ub) {
  float t = 0.5f * (lb + ub);
  for (int it = 0; it < 20; it++) {
    if (!(t >= lb && t <= ub)) t = 0.5f * (lb + ub);
    double value = quintic_eval(q, t);
    if (fabs(value) < 1e-5f || it == 19) break;
    if (value > 0.f) ub = t; else lb = t;
    double derivative = quintic_deriv(q, t);
    t = (float)(t - value / derivative);
    OPS(0, 2, 0);
  }
  return t;
}

static int within_segment(const Scene *S, int s, int seg, v2 pt, float r) {
  int so = SI(S, s, DVG_SHAPE_SEG_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS), th = SI(S, s, DVG_SHAPE_THICKNESS_OFF);
  int nc = S->d->segment_ctrl[so + seg], i0 = S->seg_point[so + seg];
  const float *P = S->P;
  if (nc == 0) {
    int i1 = (i0 + 1) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1);
    float t = dot2(sub2(pt, p0), sub2(p1, p0)) / dot2(sub2(p1, p0), sub2(p1, p0));
    float r0 = r, r1 = r;
    if (th >= 0) { r0 = P[th + i0]; r1 = P[th + i1]; }
    OPS(17, 0, 0);
    if (t < 0) return distsq2(p0, pt) < r0 * r0 ? 1 : 0;
    if (t > 1) return distsq2(p1, pt) < r1 * r1 ? 1 : 0;
    OPS(9, 0, 0);
    float rr = r0 + t * (r1 - r0);
    return distsq2(add2(p0, scl2(t, sub2(p1, p0))), pt) < rr * rr ? 1 : 0;
  } else if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1), p2 = path_pt(S, s, i2);
    if (SI(S, s, DVG_SHAPE_FLAGS) & 2) {
      v2 cp = quad_closest_approx(p0, p1, p2, pt, NULL);
      OPS(46, 0, 0);
      return distsq2(cp, pt) < r * r ? 1 : -1; /* -1: the reference returns false for the whole path */
    }
    float r0 = r, r1 = r, r2 = r;
    if (th >= 0) { r0 = P[th + i0]; r1 = P[th + i1]; r2 = P[th + i2]; }
    OPS(6, 0, 0);
    if (distsq2(eval_quad(p0, p1, p2, 0), pt) < r0 * r0) return 1;
    OPS(6, 0, 0);
    if (distsq2(eval_quad(p0, p1, p2, 1), pt) < r2 * r2) return 1;
    OPS(34, 0, 0);
    v2 v = add2(sub2(p0, scl2(2, p1)), p2), w = add2(neg2(p0), p1);
    float A = sum2(mul2(v, v));
    float B = sum2(mul2(scl2(3, v), w));
    float C = sum2(add2(mul2(scl2(2, w), w), mul2(v, sub2(p0, pt))));
    float D = sum2(mul2(w, sub2(p0, pt)));
    float t[3];
    int n = solve_cubic_f(A, B, C, D, t);
    for (int j = 0; j < n; j++) {
      if (t[j] >= 0 && t[j] <= 1) {
        OPS(16, 0, 0);
        float tt = 1 - t[j];
        float rr = (tt * tt) * r0 + (2 * tt * t[j]) * r1 + (t[j] * t[j]) * r2;
        if (distsq2(eval_quad(p0, p1, p2, t[j]), pt) < rr * rr) return 1;
      }
    }
    return 0;
  } else {
    int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1), p2 = path_pt(S, s, i2), p3 = path_pt(S, s, i3);
    float r0 = r, r1 = r, r2 = r, r3 = r;
    if (th >= 0) { r0 = P[th + i0]; r1 = P[th + i1]; r2 = P[th + i2]; r3 = P[th + i3]; }
    OPS(6, 0, 0);
    if (distsq2(eval_cubic(p0, p1, p2, p3, 0), pt) < r0 * r0) return 1;
    OPS(6, 0, 0);
    if (distsq2(eval_cubic(p0, p1, p2, p3, 1), pt) < r3 * r3) return 1;
    Quintic q = cubic_quintic(p0, p1, p2, p3, pt);
    float iv[4];
    int ni = quintic_intervals(&q, iv);
    float lower = 0.f;
    for (int j = 0; j < ni + 1; j++) {
      if (j < ni && iv[j] < 0.f) continue;
      float upper = j < ni ? rmin(iv[j], 1.f) : 1.f;
      float lb = lower, ub = upper;
      double lbe = quintic_eval(&q, lb), ube = quintic_eval(&q, ub);
      OPS(0, 1, 0);
      if (lbe * ube > 0) continue;
      if (lbe > ube) { float tmp = lb; lb = ub; ub = tmp; }
      float t = quintic_root(&q, lb, ub);
      OPS(21, 0, 0);
      float tt = 1 - t;
      float rr = (tt * tt * tt) * r0 + (3 * tt * tt * t) * r1 + (3 * tt * t * t) * r2 + (t * t * t) * r3;
      if (distsq2(eval_cubic(p0, p1, p2, p3, t), pt) < rr * rr) return 1;
      if (upper >= 1.f) break;
      lower = upper;
    }
    return 0;
  }
}

static int within_shape(const Scene *S, int s, v2 pt, float r) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  const float *p = S->P + SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    float dc = dist2(V2(p[1], p[2]), pt);
    return fabsf(dc - p[0]) < r;
  } else if (kind == DVG_ELLIPSE) {
    worker_fail(DVG_ERR_UNSUPPORTED); /* within_distance.h:343-345 asserts */
    return 0;
  } else if (kind == DVG_RECT) {
    v2 lt = V2(p[0], p[1]), rt = V2(p[2], p[1]), lb = V2(p[0], p[3]), rb = V2(p[2], p[3]);
    v2 e0[4] = {lt, lt, rt, lb}, e1[4] = {lb, rt, rb, rb};
    for (int k = 0; k < 4; k++) {
      v2 a = e0[k], b = e1[k];
      float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
      if (t < 0) { if (distsq2(a, pt) < r * r) return 1; }
      else if (t > 1) { if (distsq2(b, pt) < r * r) return 1; }
      else { if (distsq2(add2(a, scl2(t, sub2(b, a))), pt) < r * r) return 1; }
    }
    return 0;
  } else {
    int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
    for (int k = 0; k < nseg; k++) {
      int seg = S->seg_order[so + k];
      if (nseg > 1 && !box_in_r(S->seg_box[so + seg], pt, S->seg_r[so + seg])) continue;
      int h = within_segment(S, s, seg, pt, r);
      if (h == 1) return 1;
      if (h == -1) return 0;
    }
    return 0;
  }
}

/* within_distance(scene, group, pt, edge_query) (within_distance.h:355-446) */
static int group_stroke(const Scene *S, int g, v2 pt, EdgeQ *eq) {
  v2 lp = xform_pt(S->c2s + 9 * g, pt);
  OPS(14, 0, 0);
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  int ret = 0;
  for (int k = 0; k < nsh; k++) {
    int s = S->d->group_shapes[off + k];
    float r = stroke_width(S, s);
    if (nsh > 1 && !box_in_r(S->s_box[s], lp, r)) continue;
    if (within_shape(S, s, lp, r)) {
      if (!eq || eq->group != g) return 1;
      ret = 1;
      if (s == eq->shape) eq->hit = 1;
    }
  }
  return ret;
}

/* ------------------------------------------------------------------------ */
/* closest point / distance (compute_distance.h:12-439)                      */
/* ------------------------------------------------------------------------ */
typedef struct { int base_point_id, point_id; float t_root; } PathInfo;

static int closest_path(const Scene *S, int s, v2 pt, float max_radius, PathInfo *info, v2 *result) {
  int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
  float min_dist = max_radius;
  v2 ret = V2(0, 0);
  int found = 0;
  for (int k = 0; k < nseg; k++) {
    int seg = S->seg_order[so + k];
    if (nseg > 1 && !box_in_r(S->seg_box[so + seg], pt, min_dist)) continue;
    int nc = S->d->segment_ctrl[so + seg], i0 = S->seg_point[so + seg];
    float dist = 0.f, t_root = 0.f;
    v2 cp = V2(0, 0);
    if (nc == 0) {
      v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, (i0 + 1) % np);
      float t = dot2(sub2(pt, p0), sub2(p1, p0)) / dot2(sub2(p1, p0), sub2(p1, p0));
      OPS(16, 0, 1);
      if (t >= 0 && t <= 1) OPS(12, 0, 0);
      if (t < 0) { dist = dist2(p0, pt); cp = p0; t_root = 0; }
      else if (t > 1) { dist = dist2(p1, pt); cp = p1; t_root = 1; }
      else { dist = dist2(add2(p0, scl2(t, sub2(p1, p0))), pt); cp = add2(p0, scl2(t, sub2(p1, p0))); t_root = t; }
    } else if (nc == 1) {
      v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, (i0 + 2) % np);
      if (SI(S, s, DVG_SHAPE_FLAGS) & 2) {
        cp = quad_closest_approx(p0, p1, p2, pt, &t_root);
        dist = dist2(cp, pt);
        OPS(45, 0, 1);
      } else {
        v2 pt0 = eval_quad(p0, p1, p2, 0), pt1 = eval_quad(p0, p1, p2, 1);
        float d0 = dist2(pt0, pt), d1 = dist2(pt1, pt);
        OPS(44, 0, 2);
        dist = d0; cp = pt0; t_root = 0;
        if (d1 < dist) { dist = d1; cp = pt1; t_root = 1; }
        v2 v = add2(sub2(p0, scl2(2, p1)), p2), w = add2(neg2(p0), p1);
        float A = sum2(mul2(v, v));
        float B = sum2(mul2(scl2(3, v), w));
        float C = sum2(add2(mul2(scl2(2, w), w), mul2(v, sub2(p0, pt))));
        float D = sum2(mul2(w, sub2(p0, pt)));
        float t[3];
        int n = solve_cubic_f(A, B, C, D, t);
        for (int j = 0; j < n; j++) {
          if (t[j] >= 0 && t[j] <= 1) {
            v2 p = eval_quad(p0, p1, p2, t[j]);
            float dp = dist2(p, pt);
            OPS(5, 0, 1);
            if (dp < dist) { dist = dp; cp = p; t_root = t[j]; }
          }
        }
      }
    } else {
      v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i0 + 1), p2 = path_pt(S, s, i0 + 2), p3 = path_pt(S, s, (i0 + 3) % np);
      v2 pt0 = eval_cubic(p0, p1, p2, p3, 0), pt1 = eval_cubic(p0, p1, p2, p3, 1);
      float d0 = dist2(pt0, pt), d1 = dist2(pt1, pt);
      OPS(10, 0, 2);
      dist = d0; cp = pt0; t_root = 0;
      if (d1 < dist) { dist = d1; cp = pt1; t_root = 1; }
      Quintic q = cubic_quintic(p0, p1, p2, p3, pt);
      float iv[4];
      int ni = quintic_intervals(&q, iv);
      float lower = 0.f;
      for (int j = 0; j < ni + 1; j++) {
        if (j < ni && iv[j] < 0.f) continue;
        float upper = j < ni ? rmin(iv[j], 1.f) : 1.f;
        float lb = lower, ub = upper;
        double lbe = quintic_eval(&q, lb), ube = quintic_eval(&q, ub);
        OPS(0, 1, 0);
        if (lbe * ube > 0) continue;
        if (lbe > ube) { float tmp = lb; lb = ub; ub = tmp; }
        float t = quintic_root(&q, lb, ub);
        v2 p = eval_cubic(p0, p1, p2, p3, t);
        float dp = dist2(p, pt);
        OPS(5, 0, 1);
        if (dp < dist) { dist = dp; cp = p; t_root = t; }
        if (upper >= 1.f) break;
        lower = upper;
      }
    }
    if (dist < min_dist) {
      min_dist = dist; ret = cp;
      info->base_point_id = seg; info->point_id = i0; info->t_root = t_root;
      found = 1;
    }
  }
  *result = ret;
  return found;
}

static int closest_shape(const Scene *S, int s, v2 pt, float max_radius, PathInfo *info, v2 *result) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  const float *p = S->P + SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    /* compute_distance.h:18-24: computes the point but reports "not found" */
    *result = add2(V2(p[1], p[2]), scl2(p[0], normalize2(sub2(pt, V2(p[1], p[2])))));
    return 0;
  } else if (kind == DVG_ELLIPSE) {
    worker_fail(DVG_ERR_UNSUPPORTED); /* compute_distance.h:362-365 asserts */
    return 0;
  } else if (kind == DVG_RECT) {
    v2 lt = V2(p[0], p[1]), rt = V2(p[2], p[1]), lb = V2(p[0], p[3]), rb = V2(p[2], p[3]);
    v2 e0[4] = {lt, lt, rt, lb}, e1[4] = {lb, rt, rb, rb};
    float min_dist = 0.f;
    v2 cp = V2(0, 0);
    for (int k = 0; k < 4; k++) {
      v2 a = e0[k], b = e1[k];
      int first = (k == 0);
      float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
      if (t < 0) { float dd = dist2(a, pt); if (first || dd < min_dist) { min_dist = dd; cp = a; } }
      else if (t > 1) { float dd = dist2(b, pt); if (first || dd < min_dist) { min_dist = dd; cp = b; } }
      else {
        /* compute_distance.h:333-338 stores p0, not the projection */
        float dd = dist2(add2(a, scl2(t, sub2(b, a))), pt);
        if (first || dd < min_dist) { min_dist = dd; cp = a; }
      }
    }
    *result = cp;
    return 1;
  }
  return closest_path(S, s, pt, max_radius, info, result);
}

/* compute_distance (compute_distance.h:373-439) */
static int group_distance(const Scene *S, int g, v2 pt, float max_radius, int *min_shape, v2 *closest,
                          PathInfo *info, float *result) {
  v2 lp = xform_pt(S->c2s + 9 * g, pt);
  OPS(14, 0, 0);
  const float *s2c = S->P + GI(S, g, DVG_GROUP_XFORM_OFF);
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  float min_dist = max_radius;
  int found = 0;
  for (int k = 0; k < nsh; k++) {
    int s = S->d->group_shapes[off + k];
    if (nsh > 1 && !box_in_r(S->s_box[s], lp, max_radius)) continue;
    PathInfo li; li.base_point_id = -1; li.point_id = -1; li.t_root = 0;
    v2 lcp = V2(0, 0);
    if (closest_shape(S, s, lp, max_radius, &li, &lcp)) {
      v2 cp = xform_pt(s2c, lcp);
      float dist = dist2(cp, pt);
      OPS(19, 0, 1);
      if (!found || dist < min_dist) {
        found = 1; min_dist = dist;
        if (min_shape) *min_shape = s;
        if (closest) *closest = cp;
        if (info) *info = li;
      }
    }
  }
  *result = min_dist;
  return found;
}

/* ------------------------------------------------------------------------ */
/* gradient accumulation helpers                                             */
/* ------------------------------------------------------------------------ */
typedef struct {
  float *dp;        /* d_params (thread-private) */
  float d_filter;   /* thread-private d filter radius */
} Grad;
static inline void gadd(Grad *G, int off, float v) { if (G && G->dp) G->dp[off] += v; }

static void atomic_addf(float *p, float v) {
  _Atomic uint32_t *a = (_Atomic uint32_t *)p;
  uint32_t old = atomic_load(a), nw;
  do {
    union { uint32_t u; float f; } o, n;
    o.u = old; n.f = o.f + v; nw = n.u;
  } while (!atomic_compare_exchange_weak(a, &old, nw));
}

/* d_length (vector.h:496-503) */
static inline v2 d_length2(v2 v, float d_l) {
  float l = sqrtf(lensq2(v));
  float d_l_sq = 0.5f * d_l / l;
  return scl2(2 * d_l_sq, v);
}
/* d_normalize (vector.h:591-601) */
static inline v2 d_normalize2(v2 v, v2 d_n) {
  float l = len2(v);
  v2 n = div2s(v, l);
  v2 dv = div2s(d_n, l);
  float d_l = -dot2(d_n, n) / l;
  return add2(dv, d_length2(v, d_l));
}

/* ------------------------------------------------------------------------ */
/* paint (diffvg.cpp:276-504)                                                */
/* ------------------------------------------------------------------------ */
static v4 stop_color(const float *c, int i) { return V4(c[4 * i], c[4 * i + 1], c[4 * i + 2], c[4 * i + 3]); }

static v4 paint_color(const Scene *S, int kind, int off, int nstops, v2 pt) {
  const float *c = S->P + off;
  if (kind == DVG_CONSTANT) return V4(c[0], c[1], c[2], c[3]);
  float t;
  if (kind == DVG_LINEAR) {
    v2 beg = V2(c[0], c[1]), end = V2(c[2], c[3]);
    t = dot2(sub2(pt, beg), sub2(end, beg)) / rmax(dot2(sub2(end, beg), sub2(end, beg)), 1e-3f);
    OPS(11, 0, 0);
  } else {
    OPS(7, 0, 1);
    v2 cen = V2(c[0], c[1]), rad = V2(c[2], c[3]);
    v2 off2 = sub2(pt, cen);
    v2 no = V2(off2.x / rad.x, off2.y / rad.y);
    t = len2(no);
  }
  const float *offs = c + 4, *cols = c + 4 + nstops;
  if (t < offs[0]) return stop_color(cols, 0);
  for (int i = 0; i < nstops - 1; i++) {
    float oc = offs[i], on = offs[i + 1];
    if (t >= oc && t < on) {
      v4 cc = stop_color(cols, i), cn = stop_color(cols, i + 1);
      float tt = (t - oc) / (on - oc);
      OPS(16, 0, 0);
      return add4(scl4(1 - tt, cc), scl4(tt, cn));
    }
  }
  return stop_color(cols, nstops - 1);
}

static void d_paint_color(const Scene *S, int kind, int off, int nstops, v2 pt, v4 d_color, Grad *G, float *d_translation) {
  const float *c = S->P + off;
  if (kind == DVG_CONSTANT) {
    gadd(G, off + 0, d_color.x); gadd(G, off + 1, d_color.y); gadd(G, off + 2, d_color.z); gadd(G, off + 3, d_color.w);
    return;
  }
  const float *offs = c + 4, *cols = c + 4 + nstops;
  int oo = off + 4, co = off + 4 + nstops;
  float t;
  v2 beg = V2(0, 0), end = V2(0, 0), cen = V2(0, 0), rad = V2(0, 0), no = V2(0, 0), off2 = V2(0, 0);
  if (kind == DVG_LINEAR) {
    beg = V2(c[0], c[1]); end = V2(c[2], c[3]);
    t = dot2(sub2(pt, beg), sub2(end, beg)) / rmax(dot2(sub2(end, beg), sub2(end, beg)), 1e-3f);
    OPS(11, 0, 0);
  } else {
    OPS(7, 0, 1);
    cen = V2(c[0], c[1]); rad = V2(c[2], c[3]);
    off2 = sub2(pt, cen);
    no = V2(off2.x / rad.x, off2.y / rad.y);
    t = len2(no);
  }
  if (t < offs[0]) {
    gadd(G, co + 0, d_color.x); gadd(G, co + 1, d_color.y); gadd(G, co + 2, d_color.z); gadd(G, co + 3, d_color.w);
    return;
  }
  for (int i = 0; i < nstops - 1; i++) {
    float oc = offs[i], on = offs[i + 1];
    if (t >= oc && t < on) {
      v4 cc = stop_color(cols, i), cn = stop_color(cols, i + 1);
      float tt = (t - oc) / (on - oc);
      OPS(28, 0, 0);
      v4 dcc = scl4(1 - tt, d_color), dcn = scl4(tt, d_color);
      v4 diff = sub4(cn, cc);
      float d_tt = d_color.x * diff.x + d_color.y * diff.y + d_color.z * diff.z + d_color.w * diff.w;
      float d_on = -d_tt * tt / (on - oc);
      float d_oc = d_tt * ((tt - 1.f) / (on - oc));
      float d_t = d_tt / (on - oc);
      gadd(G, co + 4 * i + 0, dcc.x); gadd(G, co + 4 * i + 1, dcc.y); gadd(G, co + 4 * i + 2, dcc.z); gadd(G, co + 4 * i + 3, dcc.w);
      gadd(G, co + 4 * (i + 1) + 0, dcn.x); gadd(G, co + 4 * (i + 1) + 1, dcn.y);
      gadd(G, co + 4 * (i + 1) + 2, dcn.z); gadd(G, co + 4 * (i + 1) + 3, dcn.w);
      gadd(G, oo + i, d_oc); gadd(G, oo + i + 1, d_on);
      if (kind == DVG_LINEAR) {
        OPS(34, 0, 0);
        float l = rmax(dot2(sub2(end, beg), sub2(end, beg)), 1e-3f);
        v2 d_beg = div2s(scl2(d_t, sub2(neg2(sub2(pt, beg)), sub2(end, beg))), l);
        v2 d_end = div2s(scl2(d_t, sub2(pt, beg)), l);
        float d_l = -d_t * t / l;
        if (dot2(sub2(end, beg), sub2(end, beg)) > 1e-3f) {
          d_beg = add2(d_beg, scl2(2 * d_l, sub2(beg, end)));
          d_end = add2(d_end, scl2(2 * d_l, sub2(end, beg)));
        }
        gadd(G, off + 0, d_beg.x); gadd(G, off + 1, d_beg.y); gadd(G, off + 2, d_end.x); gadd(G, off + 3, d_end.y);
        if (d_translation) { d_translation[0] += d_beg.x + d_end.x; d_translation[1] += d_beg.y + d_end.y; }
        return;
      } else {
        OPS(20, 0, 1);
        v2 d_no = d_length2(no, d_t);
        v2 d_off = V2(d_no.x / rad.x, d_no.y / rad.y);
        v2 d_rad = V2(-d_no.x * off2.x / (rad.x * rad.x), -d_no.y * off2.y / (rad.y * rad.y));
        v2 d_cen = neg2(d_off);
        gadd(G, off + 0, d_cen.x); gadd(G, off + 1, d_cen.y); gadd(G, off + 2, d_rad.x); gadd(G, off + 3, d_rad.y);
        if (d_translation) { d_translation[0] += d_cen.x; d_translation[1] += d_cen.y; }
        /* diffvg.cpp:491-498: no return here, the loop continues and the
         * last stop also receives d_color */
      }
    }
  }
  int last = co + 4 * (nstops - 1);
  gadd(G, last + 0, d_color.x); gadd(G, last + 1, d_color.y); gadd(G, last + 2, d_color.z); gadd(G, last + 3, d_color.w);
}

/* ------------------------------------------------------------------------ */
/* d_closest_point / d_compute_distance (compute_distance.h:442-949)         */
/* ------------------------------------------------------------------------ */
static void d_closest_path(const Scene *S, int s, v2 pt, v2 d_cp, const PathInfo *info, Grad *G, v2 *d_pt) {
  int np = SI(S, s, DVG_SHAPE_NUM_POINTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  int bp = info->base_point_id, i0 = info->point_id;
  int nc = S->d->segment_ctrl[so + bp];
  float t = info->t_root;
  if (nc == 0) {
    int i1 = (i0 + 1) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1);
    float tl = dot2(sub2(pt, p0), sub2(p1, p0)) / dot2(sub2(p1, p0), sub2(p1, p0));
    OPS(20, 0, 0);
    v2 d0 = V2(0, 0), d1 = V2(0, 0);
    if (tl < 0) d0 = add2(d0, d_cp);
    else if (tl > 1) d1 = add2(d1, d_cp);
    else { d0 = add2(d0, scl2(1 - tl, d_cp)); d1 = add2(d1, scl2(tl, d_cp)); }
    gadd(G, po + 2 * i0, d0.x); gadd(G, po + 2 * i0 + 1, d0.y);
    gadd(G, po + 2 * i1, d1.x); gadd(G, po + 2 * i1 + 1, d1.y);
  } else if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1), p2 = path_pt(S, s, i2);
    v2 d0 = V2(0, 0), d2 = V2(0, 0);
    if (t == 0) d0 = add2(d0, d_cp);
    else if (t == 1) d2 = add2(d2, d_cp);
    else {
      /* compute_distance.h:525-580: the control-point adjoints are written to
       * block-local shadows and discarded; only d_pt survives. */
      v2 v = add2(sub2(p0, scl2(2, p1)), p2), w = add2(neg2(p0), p1);
      float A = sum2(mul2(v, v));
      float B = sum2(mul2(scl2(3, v), w));
      float C = sum2(add2(mul2(scl2(2, w), w), mul2(v, sub2(p0, pt))));
      v2 d_p = d_cp;
      OPS(45, 0, 0);
      float tt = 1 - t;
      float d_tt = 2 * tt * dot2(d_p, p0) + 2 * t * dot2(d_p, p1);
      float d_t = -d_tt + 2 * tt * dot2(d_p, p1) + 2 * t * dot2(d_p, p2);
      float pd = 3 * A * t * t + 2 * B * t + C;
      if (fabsf(pd) > 1e-6f) {
        float d_C = -(d_t / pd) * t;
        float d_D = -(d_t / pd);
        *d_pt = add2(*d_pt, add2(scl2(d_C, neg2(v)), scl2(d_D, neg2(w))));
      }
    }
    gadd(G, po + 2 * i0, d0.x); gadd(G, po + 2 * i0 + 1, d0.y);
    gadd(G, po + 2 * i2, d2.x); gadd(G, po + 2 * i2 + 1, d2.y);
  } else {
    int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1), p2 = path_pt(S, s, i2), p3 = path_pt(S, s, i3);
    /* double-valued accumulators: the float += double updates of the
     * reference round after every term, kept here by the casts below */
    v2 d0 = V2(0, 0), d1 = V2(0, 0), d2 = V2(0, 0), d3 = V2(0, 0);
    if (t == 0) d0 = add2(d0, d_cp);
    else if (t == 1) d3 = add2(d3, d_cp);
    else {
      Quintic q = cubic_quintic(p0, p1, p2, p3, pt);
      double A = (double)(3 * sum2(mul2(add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3),
                                         add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3))));
      v2 d_p = d_cp;
      OPS(84, 0, 0);
      float tt = 1 - t;
      float d_tt = 3 * tt * tt * dot2(d_p, p0) + 6 * tt * t * dot2(d_p, p1) + 3 * t * t * dot2(d_p, p2);
      float d_t = -d_tt + 3 * tt * tt * dot2(d_p, p1) + 6 * tt * t * dot2(d_p, p2) + 3 * t * t * dot2(d_p, p3);
      d0 = add2(d0, scl2(tt * tt * tt, d_p));
      d1 = add2(d1, scl2(3 * tt * tt * t, d_p));
      d2 = add2(d2, scl2(3 * tt * t * t, d_p));
      d3 = add2(d3, scl2(t * t * t, d_p));
      double pd = quintic_deriv(&q, t);
      if (fabs(pd) > 1e-10f) {
        OPS(70, 115, 0);
        double dB = -(d_t / pd) * t * t * t * t;
        double dC = -(d_t / pd) * t * t * t;
        double dD = -(d_t / pd) * t * t;
        double dE = -(d_t / pd) * t;
        double dF = -(d_t / pd);
        double dA = -dB * q.B / A - dC * q.C / A - dD * q.D / A - dE * q.E / A - dF * q.F / A;
        dB /= A; dC /= A; dD /= A; dE /= A; dF /= A;
        v2 a = add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3);
        v2 b = add2(sub2(scl2(3, p0), scl2(6, p1)), scl2(3, p2));
        v2 c = add2(scl2(-3, p0), scl2(3, p1));
        v2 e = sub2(p0, pt);
#define ACC(dst, sc, vec) do { (dst).x = (float)((double)(dst).x + (sc) * (double)(vec).x); \
                               (dst).y = (float)((double)(dst).y + (sc) * (double)(vec).y); } while (0)
        ACC(d0, dA * 3 * (-1) * 2, a);
        ACC(d1, dA * 3 * 3 * 2, a);
        ACC(d2, dA * 3 * (-3) * 2, a);
        ACC(d3, dA * 3 * 1 * 2, a);
        ACC(d0, dB * 5, add2(scl2(-1, b), scl2(3, a)));
        ACC(d1, dB * 5, add2(scl2(3, b), scl2(-6, a)));
        ACC(d2, dB * 5, add2(scl2(-3, b), scl2(3, a)));
        ACC(d3, dB * 5, b);
        {
          v2 t0 = add2(scl2(-1, c), scl2(-3, a));
          v2 t1 = scl2(3 * 2, b);
          d0.x = (float)((double)d0.x + (dC * 4 * (double)t0.x + dC * 2 * (double)t1.x));
          d0.y = (float)((double)d0.y + (dC * 4 * (double)t0.y + dC * 2 * (double)t1.y));
          t0 = add2(scl2(3, c), scl2(3, a)); t1 = scl2(-6 * 2, b);
          d1.x = (float)((double)d1.x + (dC * 4 * (double)t0.x + dC * 2 * (double)t1.x));
          d1.y = (float)((double)d1.y + (dC * 4 * (double)t0.y + dC * 2 * (double)t1.y));
          t0 = scl2(-3, c); t1 = scl2(3 * 2, b);
          d2.x = (float)((double)d2.x + (dC * 4 * (double)t0.x + dC * 2 * (double)t1.x));
          d2.y = (float)((double)d2.y + (dC * 4 * (double)t0.y + dC * 2 * (double)t1.y));
          ACC(d3, dC * 4, c);
        }
        {
          v2 t0 = add2(scl2(3, c), scl2(-3, b));
          v2 t1 = add2(scl2(-1, e), scl2(1, a));
          d0.x = (float)((double)d0.x + (dD * 3 * (double)t0.x + dD * 3 * (double)t1.x));
          d0.y = (float)((double)d0.y + (dD * 3 * (double)t0.y + dD * 3 * (double)t1.y));
          t0 = add2(scl2(-6, c), scl2(3, b)); t1 = scl2(3, e);
          d1.x = (float)((double)d1.x + (dD * 3 * (double)t0.x + dD * 3 * (double)t1.x));
          d1.y = (float)((double)d1.y + (dD * 3 * (double)t0.y + dD * 3 * (double)t1.y));
          t0 = scl2(3, c); t1 = scl2(-3, e);
          d2.x = (float)((double)d2.x + (dD * 3 * (double)t0.x + dD * 3 * (double)t1.x));
          d2.y = (float)((double)d2.y + (dD * 3 * (double)t0.y + dD * 3 * (double)t1.y));
          ACC(*d_pt, dD * 3, scl2(-1, a));
        }
        {
          v2 t0 = scl2(-3 * 2, c);
          v2 t1 = add2(scl2(1, b), scl2(3, e));
          d0.x = (float)((double)d0.x + (dE * (double)t0.x + dE * 2 * (double)t1.x));
          d0.y = (float)((double)d0.y + (dE * (double)t0.y + dE * 2 * (double)t1.y));
          t0 = scl2(3 * 2, c); t1 = scl2(-6, e);
          d1.x = (float)((double)d1.x + (dE * (double)t0.x + dE * 2 * (double)t1.x));
          d1.y = (float)((double)d1.y + (dE * (double)t0.y + dE * 2 * (double)t1.y));
          ACC(d2, dE * 2, scl2(3, e));
          ACC(*d_pt, dE * 2, scl2(-1, b));
        }
        {
          v2 t0 = scl2(1, c), t1 = scl2(-3, e);
          d0.x = (float)((double)d0.x + (dF * (double)t0.x + dF * (double)t1.x));
          d0.y = (float)((double)d0.y + (dF * (double)t0.y + dF * (double)t1.y));
          ACC(d1, dF, scl2(3, e));
          ACC(*d_pt, dF, scl2(-1, c));
        }
#undef ACC
      }
    }
    gadd(G, po + 2 * i0, d0.x); gadd(G, po + 2 * i0 + 1, d0.y);
    gadd(G, po + 2 * i1, d1.x); gadd(G, po + 2 * i1 + 1, d1.y);
    gadd(G, po + 2 * i2, d2.x); gadd(G, po + 2 * i2 + 1, d2.y);
    gadd(G, po + 2 * i3, d3.x); gadd(G, po + 2 * i3 + 1, d3.y);
  }
}

static void d_closest_rect(const float *p, int po, v2 pt, v2 d_cp, Grad *G, v2 *d_pt) {
  v2 lt = V2(p[0], p[1]), rt = V2(p[2], p[1]), lb = V2(p[0], p[3]), rb = V2(p[2], p[3]);
  v2 e0[4] = {lt, lt, rt, lb}, e1[4] = {lb, rt, rb, rb};
  float dd[4];
  for (int k = 0; k < 4; k++) {
    v2 a = e0[k], b = e1[k];
    float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
    if (t < 0) dd[k] = dist2(a, pt);
    else if (t > 1) dd[k] = dist2(b, pt);
    else dd[k] = dist2(add2(a, scl2(t, sub2(b, a))), pt);
  }
  int mid = 0; float md = dd[0];
  if (dd[1] < md) { md = dd[1]; mid = 1; }
  if (dd[2] < md) { md = dd[2]; mid = 2; }
  if (dd[3] < md) { md = dd[3]; mid = 3; }
  v2 dv[4] = {V2(0, 0), V2(0, 0), V2(0, 0), V2(0, 0)}; /* lt, rt, lb, rb */
  int ia[4] = {0, 0, 1, 2}, ib[4] = {2, 1, 3, 3};
  v2 a = e0[mid], b = e1[mid];
  v2 *da = &dv[ia[mid]], *db = &dv[ib[mid]];
  float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
  if (t < 0) *da = add2(*da, d_cp);
  else if (t > 1) *db = add2(*db, d_cp);
  else {
    v2 d_p = d_cp;
    *da = add2(*da, scl2(1 - t, d_p));
    *db = add2(*db, scl2(t, d_p));
    float d_t = sum2(mul2(d_p, sub2(b, a)));
    float d_num = d_t / dot2(sub2(b, a), sub2(b, a));
    float d_den = d_t * (-t) / dot2(sub2(b, a), sub2(b, a));
    *d_pt = add2(*d_pt, scl2(d_num, sub2(b, a)));
    *db = add2(*db, scl2(d_num, sub2(pt, a)));
    *da = add2(*da, scl2(d_num, add2(sub2(a, b), sub2(a, pt))));
    *db = add2(*db, scl2(d_den, scl2(2, sub2(b, a))));
    *da = add2(*da, scl2(d_den, scl2(2, sub2(a, b))));
  }
  v2 dmin = V2(0, 0), dmax = V2(0, 0);
  dmin = add2(dmin, dv[0]);
  dmax.x += dv[1].x; dmin.y += dv[1].y;
  dmin.x += dv[2].x; dmax.y += dv[2].y;
  dmax = add2(dmax, dv[3]);
  gadd(G, po + 0, dmin.x); gadd(G, po + 1, dmin.y); gadd(G, po + 2, dmax.x); gadd(G, po + 3, dmax.y);
}

static void d_closest_shape(const Scene *S, int s, v2 pt, v2 d_cp, const PathInfo *info, Grad *G, v2 *d_pt) {
  int kind = SI(S, s, DVG_SHAPE_KIND), po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  const float *p = S->P + po;
  if (kind == DVG_CIRCLE) {
    v2 c = V2(p[1], p[2]);
    v2 dn = d_normalize2(sub2(pt, c), scl2(p[0], d_cp));
    v2 d_center = mul2(d_cp, V2(1 + dn.x, 1 + dn.y));
    gadd(G, po + 1, d_center.x); gadd(G, po + 2, d_center.y);
    gadd(G, po + 0, dot2(d_cp, normalize2(sub2(pt, c))));
  } else if (kind == DVG_ELLIPSE) {
    worker_fail(DVG_ERR_UNSUPPORTED);
  } else if (kind == DVG_PATH) {
    d_closest_path(S, s, pt, d_cp, info, G, d_pt);
  } else {
    d_closest_rect(p, po, pt, d_cp, G, d_pt);
  }
}

/* 3x3 helpers for d_compute_distance (matrix.h:168-182, 244-250, 261-271) */
static void mat_mul3(const float *a, const float *b, float *r) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      float acc = 0.f;
      for (int k = 0; k < 3; k++) acc += a[3 * i + k] * b[3 * k + j];
      r[3 * i + j] = acc;
    }
}

static void d_group_distance(const Scene *S, int g, int s, v2 pt, v2 closest, const PathInfo *info, float d_dist,
                             Grad *G, float *d_translation) {
  OPS(5, 0, 0);
  if (distsq2(pt, closest) < 1e-10f) return;
  OPS(221, 0, 1);
  const float *c2s = S->c2s + 9 * g;
  int xo = GI(S, g, DVG_GROUP_XFORM_OFF);
  const float *s2c = S->P + xo;
  v2 lp = xform_pt(c2s, pt), lcp = xform_pt(c2s, closest);
  v2 d_pt = V2(0, 0), d_cp = V2(0, 0);
  {
    v2 dv = d_length2(sub2(pt, closest), d_dist); /* d_distance(closest, pt) */
    d_cp = sub2(d_cp, dv);
    d_pt = add2(d_pt, dv);
  }
  v2 d_lcp = V2(0, 0);
  float d_s2c[9] = {0};
  d_xform_pt(s2c, lcp, d_cp, d_s2c, &d_lcp);
  v2 d_lp = V2(0, 0);
  d_closest_shape(S, s, lp, d_lcp, info, G, &d_lp);
  float d_c2s[9] = {0};
  d_xform_pt(c2s, pt, d_lp, d_c2s, &d_pt);
  float t[9], nt[9], tmp[9], prod[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) t[3 * i + j] = c2s[3 * j + i];
  for (int i = 0; i < 9; i++) nt[i] = -t[i];
  mat_mul3(nt, d_c2s, tmp);
  mat_mul3(tmp, t, prod);
  for (int i = 0; i < 9; i++) d_s2c[i] += prod[i];
  for (int i = 0; i < 9; i++) gadd(G, xo + i, d_s2c[i]);
  if (d_translation) { d_translation[0] += -d_pt.x; d_translation[1] += -d_pt.y; }
}

/* ------------------------------------------------------------------------ */
/* sample_color (diffvg.cpp:525-707)                                         */
/* ------------------------------------------------------------------------ */
typedef struct { float r, g, b, a; int group; int stroke; } Frag;

static v4 sample_color(const Scene *S, const v4 *bg, v2 screen_pt, const v4 *d_color, EdgeQ *eq,
                       v4 *d_bg, float *d_translation, Grad *G, int *overflow) {
  if (eq) eq->hit = 0;
  v2 pt = V2(screen_pt.x * S->W, screen_pt.y * S->H);
  Frag frags[MAX_FRAGMENTS];
  int nf = 0, n;
  const int *cand = candidates(S, pt, &n);
  int G_ = S->d->num_groups;
  for (int k = 0; k < n; k++) {
    int g = cand[k];
    if (G_ > 1 && !box_in_r(S->g_canvas_box[g], pt, S->g_max_radius[g])) continue;
    int sk = GI(S, g, DVG_GROUP_STROKE_KIND), fk = GI(S, g, DVG_GROUP_FILL_KIND);
    if (sk != DVG_PAINT_NONE && group_stroke(S, g, pt, eq)) {
      if (nf >= MAX_FRAGMENTS) { *overflow = 1; break; }
      v4 c = paint_color(S, sk, GI(S, g, DVG_GROUP_STROKE_OFF), GI(S, g, DVG_GROUP_STROKE_STOPS), pt);
      Frag f = {c.x, c.y, c.z, c.w, g, 1};
      frags[nf++] = f;
    }
    if (fk != DVG_PAINT_NONE && group_inside(S, g, pt, eq)) {
      if (nf >= MAX_FRAGMENTS) { *overflow = 1; break; }
      v4 c = paint_color(S, fk, GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS), pt);
      Frag f = {c.x, c.y, c.z, c.w, g, 0};
      frags[nf++] = f;
    }
  }
  if (nf <= 0) {
    if (bg) {
      if (d_bg) *d_bg = *d_color;
      return *bg;
    }
    return V4(0, 0, 0, 0);
  }
  float acc_r[MAX_FRAGMENTS], acc_g[MAX_FRAGMENTS], acc_b[MAX_FRAGMENTS], acc_a[MAX_FRAGMENTS];
  float first_a = 0.f, first_r = 0.f, first_g = 0.f, first_b = 0.f;
  if (bg) { first_a = bg->w; first_r = bg->x; first_g = bg->y; first_b = bg->z; }
  for (int i = 0; i < nf; i++) {
    const Frag *f = &frags[i];
    float na = f->a;
    float pa = i > 0 ? acc_a[i - 1] : first_a;
    float pr = i > 0 ? acc_r[i - 1] : first_r, pg = i > 0 ? acc_g[i - 1] : first_g, pb = i > 0 ? acc_b[i - 1] : first_b;
    if (eq) {
      if (na >= 1.f && eq->hit) eq->hit = 0;
      if (eq->group == f->group) eq->hit = 1;
    }
    OPS(12, 0, 0);
    acc_r[i] = pr * (1 - na) + na * f->r;
    acc_g[i] = pg * (1 - na) + na * f->g;
    acc_b[i] = pb * (1 - na) + na * f->b;
    acc_a[i] = pa * (1 - na) + na;
  }
  float fr = acc_r[nf - 1], fg = acc_g[nf - 1], fb = acc_b[nf - 1], fa = acc_a[nf - 1];
  if (fa > 1e-6f) { fr /= fa; fg /= fa; fb /= fa; OPS(3, 0, 0); }
  if (d_color) {
    float dcr = d_color->x, dcg = d_color->y, dcb = d_color->z, dca = d_color->w;
    if (fa > 1e-6f) {
      float nr = d_color->x / fa, ng = d_color->y / fa, nb = d_color->z / fa;
      dca -= (d_color->x * fr + d_color->y * fg + d_color->z * fb) / fa;
      dcr = nr; dcg = ng; dcb = nb;
    }
    for (int i = nf - 1; i >= 0; i--) {
      const Frag *f = &frags[i];
      float pa = i > 0 ? acc_a[i - 1] : first_a;
      float pr = i > 0 ? acc_r[i - 1] : first_r, pg = i > 0 ? acc_g[i - 1] : first_g, pb = i > 0 ? acc_b[i - 1] : first_b;
      OPS(21, 0, 0);
      float d_pa = dca * (1.f - f->a);
      float d_ai = dca * (1.f - pa);
      d_ai += dcr * (f->r - pr) + dcg * (f->g - pg) + dcb * (f->b - pb);
      float d_pr = dcr * (1 - f->a), d_pg = dcg * (1 - f->a), d_pb = dcb * (1 - f->a);
      v4 dci = V4(dcr * f->a, dcg * f->a, dcb * f->a, d_ai);
      int g = f->group;
      if (f->stroke)
        d_paint_color(S, GI(S, g, DVG_GROUP_STROKE_KIND), GI(S, g, DVG_GROUP_STROKE_OFF), GI(S, g, DVG_GROUP_STROKE_STOPS), pt, dci, G, d_translation);
      else
        d_paint_color(S, GI(S, g, DVG_GROUP_FILL_KIND), GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS), pt, dci, G, d_translation);
      dcr = d_pr; dcg = d_pg; dcb = d_pb; dca = d_pa;
    }
    if (d_bg) { d_bg->x += dcr; d_bg->y += dcg; d_bg->z += dcb; d_bg->w += dca; }
  }
  return V4(fr, fg, fb, fa);
}

/* smoothstep / d_smoothstep (diffvg.cpp:817-833) */
static inline float smoothstep(float d) {
  OPS(6, 0, 0);
  float t = clampf_((d + 1.f) / 2.f, 0.f, 1.f);
  return t * t * (3 - 2 * t);
}
static inline float d_smoothstep(float d, float d_ret) {
  if (d < -1.f || d > 1.f) return 0.f;
  OPS(7, 0, 0);
  float t = (d + 1.f) / 2.f;
  float d_t = d_ret * (6 * t - 6 * t * t);
  return d_t / 2.f;
}

typedef struct {
  float r, g, b, a;
  int group, stroke, shape;
  float distance;
  v2 closest;
  PathInfo info;
  int within;
} PFrag;

/* sample_color_prefiltered (diffvg.cpp:835-1113) */
static v4 sample_color_prefiltered(const Scene *S, const v4 *bg, v2 screen_pt, const v4 *d_color, v4 *d_bg,
                                   float *d_translation, Grad *G, int *overflow) {
  v2 pt = V2(screen_pt.x * S->W, screen_pt.y * S->H);
  PFrag frags[MAX_PREFILTER_FRAGMENTS];
  int nf = 0, n;
  const int *cand = candidates(S, pt, &n);
  int G_ = S->d->num_groups;
  for (int k = 0; k < n; k++) {
    int g = cand[k];
    if (G_ > 1 && !box_in_r(S->g_canvas_box[g], pt, S->g_max_radius[g])) continue;
    int sk = GI(S, g, DVG_GROUP_STROKE_KIND), fk = GI(S, g, DVG_GROUP_FILL_KIND);
    if (sk != DVG_PAINT_NONE) {
      int ms = -1; v2 cp = V2(0, 0); PathInfo li = {-1, -1, 0}; float d = INFINITY;
      group_distance(S, g, pt, INFINITY, &ms, &cp, &li, &d);
      if (ms == -1) { worker_fail(DVG_ERR_UNSUPPORTED); continue; } /* diffvg.cpp:867 asserts */
      float sw = stroke_width(S, ms);
      float w = smoothstep(fabsf(d) + sw) - smoothstep(fabsf(d) - sw);
      if (w > 0) {
        if (nf >= MAX_PREFILTER_FRAGMENTS) { *overflow = 1; break; }
        v4 c = paint_color(S, sk, GI(S, g, DVG_GROUP_STROKE_OFF), GI(S, g, DVG_GROUP_STROKE_STOPS), pt);
        PFrag f = {c.x, c.y, c.z, c.w * w, g, 1, ms, d, cp, li, 1};
        frags[nf++] = f;
      }
    }
    if (fk != DVG_PAINT_NONE) {
      int ms = -1; v2 cp = V2(0, 0); PathInfo li = {-1, -1, 0}; float d = INFINITY;
      int found = group_distance(S, g, pt, 1.f, &ms, &cp, &li, &d);
      int ins = group_inside(S, g, pt, NULL);
      if (found || ins) {
        if (!ins) d = -d;
        float w = smoothstep(d);
        if (w > 0) {
          if (nf >= MAX_PREFILTER_FRAGMENTS) { *overflow = 1; break; }
          v4 c = paint_color(S, fk, GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS), pt);
          PFrag f = {c.x, c.y, c.z, c.w * w, g, 0, ms, d, cp, li, found};
          frags[nf++] = f;
        }
      }
    }
  }
  if (nf <= 0) {
    if (bg) {
      if (d_bg) *d_bg = *d_color;
      return *bg;
    }
    return V4(0, 0, 0, 0);
  }
  float acc_r[MAX_PREFILTER_FRAGMENTS], acc_g[MAX_PREFILTER_FRAGMENTS], acc_b[MAX_PREFILTER_FRAGMENTS], acc_a[MAX_PREFILTER_FRAGMENTS];
  float first_a = 0.f, first_r = 0.f, first_g = 0.f, first_b = 0.f;
  if (bg) { first_a = bg->w; first_r = bg->x; first_g = bg->y; first_b = bg->z; }
  for (int i = 0; i < nf; i++) {
    const PFrag *f = &frags[i];
    float na = f->a;
    float pa = i > 0 ? acc_a[i - 1] : first_a;
    float pr = i > 0 ? acc_r[i - 1] : first_r, pg = i > 0 ? acc_g[i - 1] : first_g, pb = i > 0 ? acc_b[i - 1] : first_b;
    OPS(12, 0, 0);
    acc_r[i] = pr * (1 - na) + na * f->r;
    acc_g[i] = pg * (1 - na) + na * f->g;
    acc_b[i] = pb * (1 - na) + na * f->b;
    acc_a[i] = pa * (1 - na) + na;
  }
  float fr = acc_r[nf - 1], fg = acc_g[nf - 1], fb = acc_b[nf - 1], fa = acc_a[nf - 1];
  if (fa > 1e-6f) { fr /= fa; fg /= fa; fb /= fa; OPS(3, 0, 0); }
  if (d_color) {
    float dcr = d_color->x, dcg = d_color->y, dcb = d_color->z, dca = d_color->w;
    if (fa > 1e-6f) {
      float nr = d_color->x / fa, ng = d_color->y / fa, nb = d_color->z / fa;
      dca -= (d_color->x * fr + d_color->y * fg + d_color->z * fb) / fa;
      dcr = nr; dcg = ng; dcb = nb;
    }
    for (int i = nf - 1; i >= 0; i--) {
      const PFrag *f = &frags[i];
      float pa = i > 0 ? acc_a[i - 1] : first_a;
      float pr = i > 0 ? acc_r[i - 1] : first_r, pg = i > 0 ? acc_g[i - 1] : first_g, pb = i > 0 ? acc_b[i - 1] : first_b;
      OPS(21, 0, 0);
      float d_pa = dca * (1.f - f->a);
      float d_ai = dca * (1.f - pa);
      d_ai += dcr * (f->r - pr) + dcg * (f->g - pg) + dcb * (f->b - pb);
      float d_pr = dcr * (1 - f->a), d_pg = dcg * (1 - f->a), d_pb = dcb * (1 - f->a);
      float dcir = dcr * f->a, dcig = dcg * f->a, dcib = dcb * f->a;
      int g = f->group;
      if (f->stroke) {
        float d = f->distance;
        float sw = stroke_width(S, f->shape);
        float apw = fabsf(d) + sw, amw = fabsf(d) - sw;
        float w = smoothstep(apw) - smoothstep(amw);
        if (w != 0) {
          float d_w = w > 0 ? (f->a / w) * d_ai : 0.f;
          d_ai *= w;
          d_paint_color(S, GI(S, g, DVG_GROUP_STROKE_KIND), GI(S, g, DVG_GROUP_STROKE_OFF), GI(S, g, DVG_GROUP_STROKE_STOPS),
                        pt, V4(dcir, dcig, dcib, d_ai), G, d_translation);
          float d_apw = d_smoothstep(apw, d_w);
          float d_amw = -d_smoothstep(amw, d_w);
          float d_d = d_apw + d_amw;
          if (d < 0) d_d = -d_d;
          float d_sw = d_apw - d_amw;
          if (fabsf(d_d) > 1e-10f) d_group_distance(S, g, f->shape, pt, f->closest, &f->info, d_d, G, d_translation);
          gadd(G, SI(S, f->shape, DVG_SHAPE_STROKE_WIDTH_OFF), d_sw);
        }
      } else {
        float d = f->distance;
        float w = smoothstep(d);
        if (w != 0) {
          float d_w = w > 0 ? (f->a / w) * d_ai : 0.f;
          d_ai *= w;
          d_paint_color(S, GI(S, g, DVG_GROUP_FILL_KIND), GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS),
                        pt, V4(dcir, dcig, dcib, d_ai), G, d_translation);
          float d_d = d_smoothstep(d, d_w);
          if (d < 0) d_d = -d_d;
          if (fabsf(d_d) > 1e-10f && f->within)
            d_group_distance(S, g, f->shape, pt, f->closest, &f->info, d_d, G, d_translation);
        }
      }
      dcr = d_pr; dcg = d_pg; dcb = d_pb; dca = d_pa;
    }
    if (d_bg) { d_bg->x += dcr; d_bg->y += dcg; d_bg->z += dcb; d_bg->w += dca; }
  }
  return V4(fr, fg, fb, fa);
}

/* sample_distance (diffvg.cpp:709-775) */
static float sample_distance(const Scene *S, v2 screen_pt, float weight, const float *d_dist, float *d_translation, Grad *G) {
  v2 pt = V2(screen_pt.x * S->W, screen_pt.y * S->H);
  int min_g = -1, min_s = -1;
  float min_d = 0.f;
  v2 cpt = V2(0, 0);
  PathInfo minfo = {-1, -1, 0};
  for (int g = S->d->num_groups - 1; g >= 0; g--) {
    int s = -1; v2 p = V2(0, 0); PathInfo li = {-1, -1, 0}; float d = INFINITY;
    if (group_distance(S, g, pt, INFINITY, &s, &p, &li, &d)) {
      if (min_g == -1 || d < min_d) { min_d = d; min_g = g; min_s = s; cpt = p; minfo = li; }
    }
  }
  if (min_g == -1) return min_d;
  min_d *= weight;
  int ins = 0;
  if (GI(S, min_g, DVG_GROUP_FILL_KIND) != DVG_PAINT_NONE) {
    ins = group_inside(S, min_g, pt, NULL);
    if (ins) min_d = -min_d;
  }
  if (d_dist) {
    float d_abs = ins ? -(*d_dist) : (*d_dist);
    d_group_distance(S, min_g, min_s, pt, cpt, &minfo, d_abs, G, d_translation);
  }
  return min_d;
}

/* ------------------------------------------------------------------------ */
/* edge sampling (sample_boundary.h, cdf.h, diffvg.cpp:89-274, 1325-1475)    */
/* ------------------------------------------------------------------------ */
typedef struct { int base_point_id, point_id; float t; int is_stroke; } BData;

/* sample(cdf, n, u) (cdf.h:5-29) */
static int cdf_sample(const float *cdf, int n, float u, float *updated_u) {
  int lb = 0, len = n - 1 - lb;
  while (len > 0) {
    int half = len / 2, mid = lb + half;
    if (u < cdf[mid]) len = half;
    else { lb = mid + 1; len = len - half - 1; }
  }
  lb = lb < 0 ? 0 : (lb > n - 1 ? n - 1 : lb);
  if (updated_u) {
    if (lb > 0) *updated_u = (u - cdf[lb - 1]) / (cdf[lb] - cdf[lb - 1]);
    else *updated_u = u / cdf[lb];
  }
  return lb;
}

static v2 perturb(v2 ret, v2 *normal, float dir, float r) {
  if (dir != 0.f) {
    ret = add2(ret, scl2(dir * r, *normal));
    if (dir < 0) *normal = neg2(*normal);
  }
  return ret;
}

/* per-shape boundary samplers (sample_boundary.h:20-384) */
static v2 sample_shape_boundary(const Scene *S, int s, float t, v2 *normal, float *pdf, BData *bd, float dir) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  const float *p = S->P + SI(S, s, DVG_SHAPE_PARAM_OFF);
  float sr = stroke_width(S, s);
  if (kind == DVG_CIRCLE) {
    float r = p[0]; v2 c = V2(p[1], p[2]);
    OPS(19, 0, 3);
    v2 off = V2((float)(r * dcos(2 * (float)M_PI * t)), (float)(r * dsin(2 * (float)M_PI * t)));
    *normal = normalize2(off);
    *pdf /= (2 * (float)M_PI * r);
    return perturb(add2(c, off), normal, dir, sr);
  } else if (kind == DVG_ELLIPSE) {
    v2 r = V2(p[0], p[1]), c = V2(p[2], p[3]);
    OPS(30, 0, 5);
    v2 off = V2((float)(r.x * dcos(2 * (float)M_PI * t)), (float)(r.y * dsin(2 * (float)M_PI * t)));
    float dxdt = (float)(-r.x * dsin(2 * (float)M_PI * t) * 2 * (float)M_PI);
    float dydt = (float)(r.y * dcos(2 * (float)M_PI * t) * 2 * (float)M_PI);
    *normal = normalize2(V2(dydt, -dxdt));
    *pdf /= sqrtf(sq(dxdt) + sq(dydt));
    return perturb(add2(c, off), normal, dir, sr);
  } else if (kind == DVG_RECT) {
    v2 pmin = V2(p[0], p[1]), pmax = V2(p[2], p[3]);
    OPS(12, 0, 0);
    float w = pmax.x - pmin.x, h = pmax.y - pmin.y;
    *pdf /= (2 * (w + h));
    if (t <= w / (w + h)) {
      t *= (w + h) / w;
      if (t < 0.5f) {
        *normal = V2(0, -1);
        return perturb(add2(pmin, scl2(2 * t, V2(pmax.x - pmin.x, 0.f))), normal, dir, sr);
      } else {
        *normal = V2(0, 1);
        return perturb(add2(V2(pmin.x, pmax.y), scl2(2 * (t - 0.5f), V2(pmax.x - pmin.x, 0.f))), normal, dir, sr);
      }
    } else {
      t = (t - w / (w + h)) * (w + h) / h;
      if (t < 0.5f) {
        *normal = V2(-1, 0);
        return perturb(add2(pmin, scl2(2 * t, V2(0.f, pmax.y - pmin.y))), normal, dir, sr);
      } else {
        *normal = V2(1, 0);
        return perturb(add2(V2(pmax.x, pmin.y), scl2(2 * (t - 0.5f), V2(0.f, pmax.y - pmin.y))), normal, dir, sr);
      }
    }
  }
  /* path (sample_boundary.h:80-307) */
  int np = SI(S, s, DVG_SHAPE_NUM_POINTS), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
  int th = SI(S, s, DVG_SHAPE_THICKNESS_OFF);
  int closed = SI(S, s, DVG_SHAPE_FLAGS) & 1;
  const float *P = S->P;
  if (dir != 0.f && !closed) {
    float cap_length;
    if (th >= 0) cap_length = (float)M_PI * (P[th] + P[th + np - 1]);
    else cap_length = 2 * (float)M_PI * sr;
    float cap_prob = cap_length / (cap_length + S->s_length[s]);
    OPS(5, 0, 0);
    if (t < cap_prob) {
      OPS(14, 0, 3);
      t = t / cap_prob;
      *pdf *= cap_prob;
      float r0 = sr, r1 = sr;
      if (th >= 0) { r0 = P[th]; r1 = P[th + np - 1]; }
      if (dir < 0) {
        v2 p0 = path_pt(S, s, 0);
        v2 off = V2((float)(r0 * dcos(2 * (float)M_PI * t)), (float)(r0 * dsin(2 * (float)M_PI * t)));
        *normal = normalize2(off);
        *pdf /= (2 * (float)M_PI * r0);
        bd->base_point_id = 0; bd->point_id = 0; bd->t = 0;
        return add2(p0, off);
      } else {
        v2 p0 = path_pt(S, s, np - 1);
        v2 off = V2((float)(r1 * dcos(2 * (float)M_PI * t)), (float)(r1 * dsin(2 * (float)M_PI * t)));
        *normal = normalize2(off);
        *pdf /= (2 * (float)M_PI * r1);
        bd->base_point_id = nseg - 1;
        bd->point_id = np - 2 - S->d->segment_ctrl[so + nseg - 1];
        bd->t = 1;
        return add2(p0, off);
      }
    } else {
      t = (t - cap_prob) / (1 - cap_prob);
      *pdf *= (1 - cap_prob);
    }
  }
  int sid = cdf_sample(S->seg_cdf + so, nseg, t, &t);
  int i0 = S->seg_point[so + sid];
  int nc = S->d->segment_ctrl[so + sid];
  bd->base_point_id = sid; bd->point_id = i0; bd->t = t;
  if (t < -1e-3f || t > 1 + 1e-3f) { *pdf = 0; return V2(0, 0); }
  if (nc == 0) {
    int i1 = (i0 + 1) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1);
    OPS(19, 0, 1);
    v2 tan = sub2(p1, p0);
    float tl = len2(tan);
    if (tl == 0) { *pdf = 0; return V2(0, 0); }
    *normal = div2s(V2(-tan.y, tan.x), tl);
    *pdf *= S->seg_pmf[so + sid] / tl;
    v2 ret = add2(p0, scl2(t, sub2(p1, p0)));
    if (dir != 0.f) {
      float r0 = sr, r1 = sr;
      if (th >= 0) { r0 = P[th + i0]; r1 = P[th + i1]; }
      float r = r0 + t * (r1 - r0);
      ret = perturb(ret, normal, dir, r);
    }
    return ret;
  } else if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1), p2 = path_pt(S, s, i2);
    v2 tan = add2(scl2(2 * (1 - t), sub2(p1, p0)), scl2(2 * t, sub2(p2, p1)));
    OPS(32, 0, 1);
    float tl = len2(tan);
    if (tl == 0) { *pdf = 0; return V2(0, 0); }
    *normal = div2s(V2(-tan.y, tan.x), tl);
    *pdf *= S->seg_pmf[so + sid] / tl;
    v2 ret = eval_quad(p0, p1, p2, t);
    if (dir != 0.f) {
      float r0 = sr, r1 = sr, r2 = sr;
      if (th >= 0) { r0 = P[th + i0]; r1 = P[th + i1]; r2 = P[th + i2]; }
      float tt = 1 - t;
      float r = (tt * tt) * r0 + (2 * tt * t) * r1 + (t * t) * r2;
      ret = perturb(ret, normal, dir, r);
    }
    return ret;
  } else {
    int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
    v2 p0 = path_pt(S, s, i0), p1 = path_pt(S, s, i1), p2 = path_pt(S, s, i2), p3 = path_pt(S, s, i3);
    v2 tan = add2(add2(scl2(3 * sq(1 - t), sub2(p1, p0)), scl2(6 * (1 - t) * t, sub2(p2, p1))), scl2(3 * t * t, sub2(p3, p2)));
    OPS(44, 0, 1);
    float tl = len2(tan);
    if (tl == 0) { *pdf = 0; return V2(0, 0); }
    *normal = div2s(V2(-tan.y, tan.x), tl);
    *pdf *= S->seg_pmf[so + sid] / tl;
    v2 ret = eval_cubic(p0, p1, p2, p3, t);
    if (dir != 0.f) {
      float r0 = sr, r1 = sr, r2 = sr, r3 = sr;
      if (th >= 0) { r0 = P[th + i0]; r1 = P[th + i1]; r2 = P[th + i2]; r3 = P[th + i3]; }
      float tt = 1 - t;
      float r = (tt * tt * tt) * r0 + (3 * tt * tt * t) * r1 + (3 * tt * t * t) * r2 + (t * t * t) * r3;
      ret = perturb(ret, normal, dir, r);
    }
    return ret;
  }
}

/* sample_boundary(scene, ...) (sample_boundary.h:386-453) */
static v2 sample_boundary(const Scene *S, int g, int s, float t, v2 *normal, float *pdf, BData *bd) {
  *pdf = 1;
  int has_fill = GI(S, g, DVG_GROUP_FILL_KIND) != DVG_PAINT_NONE;
  int has_stroke = GI(S, g, DVG_GROUP_STROKE_KIND) != DVG_PAINT_NONE;
  int stroke = 0;
  if (has_fill && has_stroke) {
    if (t < 0.5f) { stroke = 0; t = 2 * t; *pdf = 0.5f; }
    else { stroke = 1; t = 2 * (t - 0.5f); *pdf = 0.5f; }
  } else if (has_stroke) {
    stroke = 1;
  }
  bd->is_stroke = stroke;
  float dir = 0.f;
  if (stroke) {
    if (t < 0.5f) { dir = -1.f; t = 2 * t; *pdf *= 0.5f; }
    else { dir = 1.f; t = 2 * (t - 0.5f); *pdf *= 0.5f; }
  }
  return sample_shape_boundary(S, s, t, normal, pdf, bd, dir);
}

/* accumulate_boundary_gradient (diffvg.cpp:89-274) */
static void accumulate_boundary_gradient(const Scene *S, int g, int s, float contrib, float t, v2 normal,
                                         const BData *bd, v2 local_pt, Grad *G) {
  int kind = SI(S, s, DVG_SHAPE_KIND), po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  /* the shape_to_canvas adjoint (d_xform_pt) and the control-point weights */
  OPS(40 + (kind == DVG_PATH ? 30 : kind == DVG_ELLIPSE ? 10 : 3), 0, kind == DVG_ELLIPSE ? 2 : 0);
  int th = kind == DVG_PATH ? SI(S, s, DVG_SHAPE_THICKNESS_OFF) : -1;
  int np = kind == DVG_PATH ? SI(S, s, DVG_SHAPE_NUM_POINTS) : 0;
  int so = kind == DVG_PATH ? SI(S, s, DVG_SHAPE_SEG_OFF) : 0;
  if (bd->is_stroke) {
    if (th >= 0) {
      int i0 = bd->point_id;
      float tt = bd->t;
      int nc = S->d->segment_ctrl[so + bd->base_point_id];
      if (nc == 0) {
        int i1 = (i0 + 1) % np;
        gadd(G, th + i0, (1 - tt) * contrib); gadd(G, th + i1, (tt) * contrib);
      } else if (nc == 1) {
        int i1 = i0 + 1, i2 = (i0 + 2) % np;
        gadd(G, th + i0, sq(1 - tt) * contrib); gadd(G, th + i1, (2 * (1 - tt) * tt) * contrib); gadd(G, th + i2, (tt * tt) * contrib);
      } else {
        int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
        gadd(G, th + i0, ((1 - tt) * (1 - tt) * (1 - tt)) * contrib);
        gadd(G, th + i1, 3 * sq(1 - tt) * tt * contrib);
        gadd(G, th + i2, 3 * (1 - tt) * tt * tt * contrib);
        gadd(G, th + i3, tt * tt * tt * contrib);
      }
    } else {
      gadd(G, SI(S, s, DVG_SHAPE_STROKE_WIDTH_OFF), contrib);
    }
  }
  if (kind == DVG_CIRCLE) {
    gadd(G, po + 1, normal.x * contrib); gadd(G, po + 2, normal.y * contrib);
    gadd(G, po + 0, contrib);
  } else if (kind == DVG_ELLIPSE) {
    gadd(G, po + 2, normal.x * contrib); gadd(G, po + 3, normal.y * contrib);
    gadd(G, po + 0, (float)(dcos(2 * (float)M_PI * t) * normal.x * contrib));
    gadd(G, po + 1, (float)(dsin(2 * (float)M_PI * t) * normal.y * contrib));
  } else if (kind == DVG_PATH) {
    int i0 = bd->point_id;
    float tt = bd->t;
    int nc = S->d->segment_ctrl[so + bd->base_point_id];
    if (nc == 0) {
      int i1 = (i0 + 1) % np;
      gadd(G, po + 2 * i0 + 0, (1 - tt) * normal.x * contrib); gadd(G, po + 2 * i0 + 1, (1 - tt) * normal.y * contrib);
      gadd(G, po + 2 * i1 + 0, (tt) * normal.x * contrib); gadd(G, po + 2 * i1 + 1, (tt) * normal.y * contrib);
    } else if (nc == 1) {
      int i1 = i0 + 1, i2 = (i0 + 2) % np;
      gadd(G, po + 2 * i0 + 0, sq(1 - tt) * normal.x * contrib); gadd(G, po + 2 * i0 + 1, sq(1 - tt) * normal.y * contrib);
      gadd(G, po + 2 * i1 + 0, (2 * (1 - tt) * tt) * normal.x * contrib); gadd(G, po + 2 * i1 + 1, (2 * (1 - tt) * tt) * normal.y * contrib);
      gadd(G, po + 2 * i2 + 0, (tt * tt) * normal.x * contrib); gadd(G, po + 2 * i2 + 1, (tt * tt) * normal.y * contrib);
    } else {
      int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
      float c0 = (1 - tt) * (1 - tt) * (1 - tt);
      gadd(G, po + 2 * i0 + 0, c0 * normal.x * contrib); gadd(G, po + 2 * i0 + 1, c0 * normal.y * contrib);
      gadd(G, po + 2 * i1 + 0, 3 * sq(1 - tt) * tt * normal.x * contrib); gadd(G, po + 2 * i1 + 1, 3 * sq(1 - tt) * tt * normal.y * contrib);
      gadd(G, po + 2 * i2 + 0, 3 * (1 - tt) * tt * tt * normal.x * contrib); gadd(G, po + 2 * i2 + 1, 3 * (1 - tt) * tt * tt * normal.y * contrib);
      gadd(G, po + 2 * i3 + 0, tt * tt * tt * normal.x * contrib); gadd(G, po + 2 * i3 + 1, tt * tt * tt * normal.y * contrib);
    }
  } else {
    if (normal.x == -1 && normal.y == 0) gadd(G, po + 0, -contrib);
    else if (normal.x == 1 && normal.y == 0) gadd(G, po + 2, contrib);
    else if (normal.x == 0 && normal.y == -1) gadd(G, po + 1, -contrib);
    else if (normal.x == 0 && normal.y == 1) gadd(G, po + 3, contrib);
    else worker_fail(DVG_ERR_UNSUPPORTED); /* diffvg.cpp:253-256 asserts */
  }
  float d_s2c[9] = {0};
  v2 d_local = V2(0, 0);
  int xo = GI(S, g, DVG_GROUP_XFORM_OFF);
  d_xform_pt(S->P + xo, local_pt, scl2(contrib, normal), d_s2c, &d_local);
  for (int i = 0; i < 9; i++) gadd(G, xo + i, d_s2c[i]);
}

/* ------------------------------------------------------------------------ */
/* render driver (diffvg.cpp:1115-1649)                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
  const Scene *S;
  const DvgOracleArgs *A;
  int w, h, nsx, nsy, ri;
  int ftype;
  float fr;
  float *weight;       /* [h*w] */
  v4 *samples;         /* [n] forward sample colours */
  int nthreads;
  Grad *grads;         /* [nthreads] */
  _Atomic int64_t overflow;
} Ctx;

static inline v2 sample_pos(const Ctx *C, int idx, int prefilter, int *x, int *y) {
  pcg32 rng = pcg_init(idx, C->A->seed);
  int sx = idx % C->nsx;
  int sy = (idx / C->nsx) % C->nsy;
  *x = (idx / (C->nsx * C->nsy)) % C->w;
  *y = (idx / (C->nsx * C->nsy * C->w));
  float rx = pcg_float(&rng), ry = pcg_float(&rng);
  OPS(8, 0, 0);
  if (prefilter) { rx = 0.5f; ry = 0.5f; }
  return V2(*x + ((float)sx + rx) / C->nsx, *y + ((float)sy + ry) / C->nsy);
}

typedef void (*task_fn)(Ctx *C, int tid, int64_t begin, int64_t end);
typedef struct { Ctx *C; task_fn fn; int tid; int64_t n, chunk; } Job;
static void *job_main(void *p) {
  Job *J = (Job *)p;
  int T = J->C->nthreads;
  for (int64_t c = J->tid; c * J->chunk < J->n; c += T) {
    int64_t b = c * J->chunk, e = b + J->chunk < J->n ? b + J->chunk : J->n;
    J->fn(J->C, J->tid, b, e);
  }
  return NULL;
}
static void run_parallel(Ctx *C, task_fn fn, int64_t n, int64_t chunk) {
  if (n <= 0) return;
  int T = C->nthreads;
  if (T <= 1) { Job J = {C, fn, 0, n, chunk}; job_main(&J); return; }
  pthread_t th[256];
  Job jobs[256];
  for (int t = 0; t < T; t++) {
    jobs[t].C = C; jobs[t].fn = fn; jobs[t].tid = t; jobs[t].n = n; jobs[t].chunk = chunk;
    pthread_create(&th[t], NULL, job_main, &jobs[t]);
  }
  for (int t = 0; t < T; t++) pthread_join(th[t], NULL);
}

/* weight image: per pixel sum of filter weights of the jittered samples in
 * its support (weight_kernel, diffvg.cpp:1115-1158; it never sees
 * use_prefiltering, diffvg.cpp:1525-1533) */
static void task_weight(Ctx *C, int tid, int64_t b, int64_t e) {
  (void)tid;
  PHASE(PH_WEIGHT);
  int spp = C->nsx * C->nsy;
  for (int64_t p = b; p < e; p++) {
    int px = (int)(p % C->w), py = (int)(p / C->w);
    float ws = 0.f;
    for (int ny = py - C->ri; ny <= py + C->ri; ny++) {
      if (ny < 0 || ny >= C->h) continue;
      for (int nx = px - C->ri; nx <= px + C->ri; nx++) {
        if (nx < 0 || nx >= C->w) continue;
        for (int k = 0; k < spp; k++) {
          int idx = (ny * C->w + nx) * spp + k, x, y;
          v2 pt = sample_pos(C, idx, 0, &x, &y);
          ws += filter_weight(C->ftype, C->fr, (px + 0.5f) - pt.x, (py + 0.5f) - pt.y);
        }
      }
    }
    C->weight[p] = ws;
  }
  ops_flush();
}

static v4 gather_d_color(const Ctx *C, v2 pt) {
  int x = (int)pt.x, y = (int)pt.y;
  v4 d = V4(0, 0, 0, 0);
  for (int dy = -C->ri; dy <= C->ri; dy++)
    for (int dx = -C->ri; dx <= C->ri; dx++) {
      int xx = x + dx, yy = y + dy;
      if (xx >= 0 && xx < C->w && yy >= 0 && yy < C->h) {
        float xc = xx + 0.5f, yc = yy + 0.5f;
        float fw = filter_weight(C->ftype, C->fr, xc - pt.x, yc - pt.y);
        float ws = C->weight[yy * C->w + xx];
        if (ws > 0) {
          const float *di = C->A->d_image + 4 * (yy * C->w + xx);
          OPS(11, 0, 0);
          d = add4(d, scl4(fw / ws, V4(di[0], di[1], di[2], di[3])));
        }
      }
    }
  return d;
}

/* render_kernel (diffvg.cpp:1160-1312), one sample per item */
static void task_render(Ctx *C, int tid, int64_t b, int64_t e) {
  const DvgOracleArgs *A = C->A;
  const Scene *S = C->S;
  Grad *G = &C->grads[tid];
  int spp = C->nsx * C->nsy;
  PHASE(PH_RENDER);
  for (int64_t i = b; i < e; i++) {
    int idx = (int)i, x = 0, y = 0;
    v2 pt;
    if (A->eval_positions == NULL) {
      pt = sample_pos(C, idx, A->use_prefiltering, &x, &y);
    } else {
      pt = V2(A->eval_positions[2 * idx], A->eval_positions[2 * idx + 1]);
      x = (int)pt.x; y = (int)pt.y;
    }
    v2 npt = V2(pt.x / C->w, pt.y / C->h);
    if (A->image || A->d_image) {
      v4 d_color = V4(0, 0, 0, 0);
      if (A->d_image) d_color = gather_d_color(C, pt);
      const v4 *bg = A->background ? (const v4 *)(A->background + 4 * (y * C->w + x)) : NULL;
      v4 *d_bg = A->d_background ? (v4 *)(A->d_background + 4 * (y * C->w + x)) : NULL;
      float *d_tr = A->d_translation ? A->d_translation + 2 * (y * C->w + x) : NULL;
      int of = 0;
      v4 color;
      if (A->use_prefiltering)
        color = sample_color_prefiltered(S, bg, npt, A->d_image ? &d_color : NULL, d_bg, d_tr, G, &of);
      else
        color = sample_color(S, bg, npt, A->d_image ? &d_color : NULL, NULL, d_bg, d_tr, G, &of);
      if (of) atomic_fetch_add(&C->overflow, 1);
      if (A->image) C->samples[idx] = color;
      if (A->d_image) {
        for (int dy = -C->ri; dy <= C->ri; dy++)
          for (int dx = -C->ri; dx <= C->ri; dx++) {
            int xx = x + dx, yy = y + dy;
            if (xx >= 0 && xx < C->w && yy >= 0 && yy < C->h && C->weight[yy * C->w + xx] > 0) {
              float ws = C->weight[yy * C->w + xx];
              float xc = xx + 0.5f, yc = yy + 0.5f;
              float fw = filter_weight(C->ftype, C->fr, xc - pt.x, yc - pt.y);
              const float *di = A->d_image + 4 * (yy * C->w + xx);
              v4 dp = V4(di[0], di[1], di[2], di[3]);
              float dd = dot4(dp, color);
              OPS(15, 0, 0);
              float d_weight = (dd * ws - fw * dd * (ws - fw)) / (ws * ws);
              G->d_filter += d_filter_weight(C->ftype, C->fr, xc - pt.x, yc - pt.y, d_weight);
            }
          }
      }
    }
    if (A->sdf || A->d_sdf) {
      float d_dist = 0.f;
      if (A->d_sdf) d_dist = A->eval_positions == NULL ? A->d_sdf[y * C->w + x] : A->d_sdf[idx];
      float weight = A->eval_positions == NULL ? 1.f / spp : 1.f;
      float *d_tr = A->d_translation ? A->d_translation + 2 * (y * C->w + x) : NULL;
      float dist = sample_distance(S, npt, weight, A->d_sdf ? &d_dist : NULL, d_tr, G);
      if (A->sdf) {
        if (A->eval_positions == NULL) A->sdf[y * C->w + x] += dist; /* one thread owns a pixel's samples */
        else A->sdf[idx] += dist;
      }
    }
  }
  ops_flush();
}

/* filtered colour of each pixel from the stored sample colours (the splat
 * of render_kernel, diffvg.cpp:1218-1249, gathered per pixel) */
static void task_resolve(Ctx *C, int tid, int64_t b, int64_t e) {
  (void)tid;
  PHASE(PH_RESOLVE);
  int spp = C->nsx * C->nsy;
  for (int64_t p = b; p < e; p++) {
    int px = (int)(p % C->w), py = (int)(p / C->w);
    float ws = C->weight[p];
    if (!(ws > 0)) continue;
    v4 acc = V4(0, 0, 0, 0);
    for (int ny = py - C->ri; ny <= py + C->ri; ny++) {
      if (ny < 0 || ny >= C->h) continue;
      for (int nx = px - C->ri; nx <= px + C->ri; nx++) {
        if (nx < 0 || nx >= C->w) continue;
        for (int k = 0; k < spp; k++) {
          int idx = (ny * C->w + nx) * spp + k, x, y;
          v2 pt = sample_pos(C, idx, C->A->use_prefiltering, &x, &y);
          float fw = filter_weight(C->ftype, C->fr, (px + 0.5f) - pt.x, (py + 0.5f) - pt.y);
          v4 c = C->samples[idx];
          OPS(12, 0, 0);
          acc = add4(acc, V4(fw * c.x / ws, fw * c.y / ws, fw * c.z / ws, fw * c.w / ws));
        }
      }
    }
    float *o = C->A->image + 4 * p;
    o[0] += acc.x; o[1] += acc.y; o[2] += acc.z; o[3] += acc.w;
  }
  ops_flush();
}

/* sample_boundary_kernel + render_edge_kernel (diffvg.cpp:1325-1475) */
static void task_edge(Ctx *C, int tid, int64_t b, int64_t e) {
  const DvgOracleArgs *A = C->A;
  const Scene *S = C->S;
  Grad *G = &C->grads[tid];
  PHASE(PH_EDGE);
  for (int64_t i = b; i < e; i++) {
    int idx = (int)i;
    pcg32 rng = pcg_init(idx, A->seed);
    float u = pcg_float(&rng);
    int sid = cdf_sample(S->smp_cdf, S->num_total, u, NULL);
    int s = S->smp_shape[sid], g = S->smp_group[sid];
    /* diffvg.cpp:1343 indexes the pmf by shape id */
    float pmf = s < S->num_total ? S->smp_pmf[s] : 0.f;
    if (pmf <= 0) continue;
    float pdf = 0.f;
    v2 normal = V2(0, 0);
    float t = pcg_float(&rng);
    BData bd; memset(&bd, 0, sizeof(bd));
    v2 lpt = sample_boundary(S, g, s, t, &normal, &pdf, &bd);
    if (pdf <= 0) continue;
    const float *s2c = S->P + GI(S, g, DVG_GROUP_XFORM_OFF);
    OPS(40, 0, 1);  /* the boundary point and normal to the canvas, the query points */
    v2 bpt = xform_pt(s2c, lpt);
    normal = xform_normal(S->c2s + 9 * g, normal);
    bpt.x /= S->W; bpt.y /= S->H;
    pdf = pmf * pdf;
    int bx = (int)(bpt.x * C->w), by = (int)(bpt.y * C->h);
    if (bx < 0 || bx >= C->w || by < 0 || by >= C->h) continue;
    EdgeQ qin = {g, s, 0}, qout = {g, s, 0};
    const v4 *bg = A->background ? (const v4 *)(A->background + 4 * (by * C->w + bx)) : NULL;
    int of = 0;
    v4 cin = sample_color(S, bg, sub2(bpt, scl2(1e-4f, normal)), NULL, &qin, NULL, NULL, NULL, &of);
    v4 cout = sample_color(S, bg, add2(bpt, scl2(1e-4f, normal)), NULL, &qout, NULL, NULL, NULL, &of);
    if (of) atomic_fetch_add(&C->overflow, 1);
    if (!qin.hit && !qout.hit) continue;
    if (!qin.hit) {
      normal = neg2(normal);
      v4 tmp = cin; cin = cout; cout = tmp;
    }
    v2 sbpt = V2(bpt.x * C->w, bpt.y * C->h);
    v4 dc = gather_d_color(C, sbpt);
    float norm = (float)(S->W * S->H);
    OPS(16, 0, 0);
    dc = V4(dc.x / norm, dc.y / norm, dc.z / norm, dc.w / norm);
    float contrib = dot4(sub4(cin, cout), dc) / pdf;
    accumulate_boundary_gradient(S, g, s, contrib, t, normal, &bd, lpt, G);
    if (A->d_translation) {
      atomic_addf(&A->d_translation[2 * (by * C->w + bx) + 0], normal.x * contrib);
      atomic_addf(&A->d_translation[2 * (by * C->w + bx) + 1], normal.y * contrib);
    }
  }
  ops_flush();
}

int dvg_oracle_render(const DvgSceneDesc *desc, const DvgOracleArgs *A, char *err, int err_len) {
  g_err = err; g_err_len = err_len; g_status = DVG_OK;
  if (err && err_len > 0) err[0] = 0;
  atomic_store(&g_worker_status, DVG_OK);
  if (!desc || !A || !A->params || A->width <= 0 || A->height <= 0 || A->num_samples_x <= 0 || A->num_samples_y <= 0) {
    fail(DVG_ERR_INVALID, "invalid arguments");
    return g_status;
  }
  Scene S;
  if (scene_init(&S, desc, A->params) != 0) { scene_free(&S); return g_status; }
  Ctx C;
  memset(&C, 0, sizeof(C));
  C.S = &S; C.A = A;
  C.w = A->width; C.h = A->height; C.nsx = A->num_samples_x; C.nsy = A->num_samples_y;
  C.ftype = desc->filter_type;
  C.fr = A->params[desc->filter_radius_off];
  C.ri = (int)ceilf(C.fr);
  C.nthreads = A->num_threads > 0 ? (A->num_threads > 256 ? 256 : A->num_threads) : 1;
  int64_t n_samples = (int64_t)C.w * C.h * C.nsx * C.nsy;
  int64_t n_px = (int64_t)C.w * C.h;
  C.grads = (Grad *)calloc((size_t)C.nthreads, sizeof(Grad));
  if (A->d_params) {
    for (int t = 0; t < C.nthreads; t++) C.grads[t].dp = (float *)calloc((size_t)(desc->num_params > 0 ? desc->num_params : 1), sizeof(float));
  }
  if (desc->num_groups == 0) {
    /* empty scene: background (or zero) and no gradients */
    if (A->image && A->eval_positions == NULL) {
      for (int64_t p = 0; p < n_px; p++)
        for (int c = 0; c < 4; c++) A->image[4 * p + c] += A->background ? A->background[4 * p + c] : 0.f;
    }
    goto done;
  }
  int want = A->image || A->d_image || A->sdf || A->d_sdf;
  if (want) {
    if (A->eval_positions == NULL) {
      C.weight = (float *)calloc((size_t)n_px, sizeof(float));
      run_parallel(&C, task_weight, n_px, C.w);
    }
    int64_t n = A->eval_positions == NULL ? n_samples : A->num_eval_positions;
    if (A->image) C.samples = (v4 *)calloc((size_t)(n > 0 ? n : 1), sizeof(v4));
    /* one chunk = one pixel row, so a thread owns all samples of a pixel */
    int64_t chunk = A->eval_positions == NULL ? (int64_t)C.w * C.nsx * C.nsy : 256;
    run_parallel(&C, task_render, n, chunk);
    if (A->image && A->eval_positions == NULL) run_parallel(&C, task_resolve, n_px, C.w);
  }
  if (!A->use_prefiltering && A->d_image && A->eval_positions == NULL) {
    run_parallel(&C, task_edge, n_samples, 4096);
  }
done:
  if (A->d_params) {
    for (int t = 0; t < C.nthreads; t++) {
      for (int i = 0; i < desc->num_params; i++) A->d_params[i] += C.grads[t].dp[i];
      A->d_params[desc->filter_radius_off] += C.grads[t].d_filter;
    }
  }
  if (A->counters) A->counters[0] = (int64_t)atomic_load(&C.overflow);
  for (int t = 0; t < C.nthreads; t++) free(C.grads[t].dp);
  free(C.grads); free(C.weight); free(C.samples);
  scene_free(&S);
  if (atomic_load(&C.overflow) > 0) fail(DVG_ERR_CAPACITY, "fragment list overflow");
  int ws = atomic_load(&g_worker_status);
  if (ws != DVG_OK) fail(ws, "unsupported input (the reference asserts on it): ellipse stroke/prefilter, circle stroke prefilter or rotated rect edge");
  return g_status;
}
