// Device-side scene representation and per-sample geometry of the GB300
// render path.
//
// Everything here is __device__ code evaluated per sample (or per boundary
// sample).  Arithmetic follows the reference's evaluation order and
// precision (fp32 where it computes in float, fp64 where it promotes to
// double) so that sample classification (inside / outside, within stroke or
// not) agrees with the reference CPU build; the library is compiled with
// --fmad=false for the same reason.  Each function cites the reference
// file:line whose semantics it implements.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/diffvg_gb300.h"

#define DVG_TILE 16
#define DVG_MAX_FRAGMENTS 256          // diffvg.cpp:542
#define DVG_MAX_PREFILTER_FRAGMENTS 64 // diffvg.cpp:847
#define DVG_PI 3.14159265358979323846

// error bits of the per-scene device status word
enum {
  DVG_EFLAG_CAPACITY = 1u,     // fragment list above the reference's cap
  DVG_EFLAG_UNSUPPORTED = 2u,  // input on which the reference asserts
  DVG_EFLAG_SCENE_ZERO = 4u,   // total boundary length <= 0
  DVG_EFLAG_SCENE_NAN = 8u,    // total boundary length not finite
  DVG_EFLAG_FILTER = 16u,      // filter radius outside [0, 64]
};

// Resident scene: topology (uploaded once) + per-call derived arrays.
struct DevScene {
  int W, H;  // canvas size
  int num_shapes, num_groups, num_segments, num_total;
  const int *shape_info;    // [S * DVG_SHAPE_INFO_STRIDE]
  const int *segment_ctrl;  // [NSEG]
  const int *seg_point;     // [NSEG] first point of each segment within its path
  const int *group_info;    // [G * DVG_GROUP_INFO_STRIDE]
  const int *group_shapes;  // [sum of group sizes]
  const int *smp_shape;     // [num_total] (group, shape) pairs of the boundary CDF
  const int *smp_group;
  const float *P;           // parameter arena
  // derived per call from P
  float *c2s;               // [G*9] canvas_to_shape
  float4 *g_local_box;      // [G] (lo.x, lo.y, hi.x, hi.y) in shape space
  float4 *g_canvas_box;     // [G] in canvas space
  float *g_max_radius;      // [G]
  float4 *s_box;            // [S]
  float *s_length;          // [S]
  float4 *seg_box;          // [NSEG]
  float *seg_r, *seg_pmf, *seg_cdf;
  int *seg_order;           // [NSEG] per-path visiting order (local indices)
  float *smp_cdf, *smp_pmf; // [num_total]
  int tiles_x, tiles_y;
  int *tile_start;          // [tiles+1]
  int *tile_list;           // candidate groups per tile, ascending
  unsigned *tile_mask;      // per tile-list entry: bit i set when one of the group's stroke records
                            // [i << c, (i + 1) << c) may reach the tile, c = rec_chunk_shift(records)
  int *scratch;             // [8*NSEG + 8*S] path leaf-order scratch
  int2 *g_rec;              // [G] range of each group's stroke records
  float4 *rec_box;          // [records] cull box (empty test: infinite box)
  int4 *rec_a;              // {segment (so + seg; -1: whole-shape record), shape, nc, first point}
  int4 *rec_b;              // {param offset, point count, thickness offset, first record of the next shape}
  float *rec_r;             // stroke radius of the record's shape
  float4 *rec_cbox;         // canvas box of the record's cull box (one pixel wider), for tile binning
  float2 *seg_tpts = nullptr;  // [NSEG * DVG_TREE_PTS] tabulated subdivision trees (curved segments), or null
  float *seg_th = nullptr;     // [NSEG * DVG_TREE_NODES]
  int wide_queues = 0;         // stroke-heavy scene: the walks queue DVG_LANE_JOBS_WIDE tests per lane
  int fill_heavy = 0;          // fill-heavy scene: the sampled forward runs DVG_FWD_FILL_BLOCKS blocks per SM
  int num_paths = 1, num_records = 1;  // path shapes and stroke records (preparation skips the kernels of none)
  unsigned *err;            // status word (DVG_EFLAG_*)
  // y-band segment lists of long paths (null: no path has them).  A path of
  // DVG_BAND_MIN_SEGMENTS or more segments splits its box's y-range into up
  // to shape_band.x equal bands; band b lists, in visiting order, the
  // segments whose box meets the band.  shape_band = {bands (0: none), first entry of
  // the path's band_start (bands + 1 entries), first entry of its band_seg,
  // band_seg capacity} is topology; the rest is derived per call.
  const int4 *shape_band = nullptr;  // [S]
  float2 *band_geo = nullptr;        // [S] y of the box's top, bands per unit of y
  int *band_n = nullptr;             // [S] bands in use this call (0: lists off, e.g. over capacity)
  int *band_start = nullptr;         // band b of path s: band_seg[shape_band.z + band_start[shape_band.y + b] ...]
  int *band_seg = nullptr;           // visiting ranks k of the segments (segment seg_order[k] of the path)
};
// Paths with fewer segments scan them all: a warp's lanes then walk one list
// together, which costs less than divergent walks of short band lists.
#define DVG_BAND_MIN_SEGMENTS 64
// Bands are at least this tall (shape-space units), so that a warp's pixel
// block and a prefiltering query's +-1 px range mostly fall in one band.
#define DVG_BAND_MIN_HEIGHT 4.0f

// Per-call render settings (image space).
struct DevRender {
  int w, h, nsx, nsy, spp;
  uint64_t seed;
  int prefilter;
  int ftype;
  const float *fr_ptr;       // filter radius in the parameter arena
  float fr;                  // *fr_ptr, loaded on the device (load_filter)
  int ri;                    // ceil(fr)
  const float *background;   // [h*w*4] or null
  float *weight;             // [h*w]
  const float *d_image;      // [h*w*4] or null
  float *d_params;           // gradient arena or null
  float *d_background;       // [h*w*4] or null
  float *d_translation;      // [h*w*2] or null
  int filter_radius_off;
  // fragment cache from the forward pass to the backward pass of the same
  // parameters: the keys of each sample's hit fragments in blend order
  // ([DVG_HIT_SLOTS][samples]) and their count (DVG_HIT_NONE: not cached)
  int *hit_keys = nullptr;
  void *pf_frags = nullptr;  // prefiltered: [DVG_PF_SLOTS][samples] fragments instead of keys
  unsigned short *hit_cnt = nullptr;
  const unsigned *hit_stale = nullptr;  // backward: nonzero when the parameters differ from the forward's
  // entries past the slots: without prefiltering, chunks of DVG_HIT_CHUNK
  // keys and the next chunk's index ([hit_chunk_cap][DVG_HIT_CHUNK + 1]);
  // with prefiltering, chunks of DVG_PF_CHUNK fragments (pf_chunk_frags)
  // and the next chunk's index ([hit_chunk_cap]); each sample's first chunk
  // ([samples]) and the count of chunks handed out
  int *hit_chunks = nullptr;
  void *pf_chunk_frags = nullptr;
  int *hit_first = nullptr;
  int *hit_chunk_count = nullptr;
  int hit_chunk_cap = 0;
  // backward: the samples left to the deep pass ([samples]) and their count
  int *deep_list = nullptr;
  int *deep_count = nullptr;
};
#define DVG_HIT_SLOTS 16
#define DVG_HIT_NONE 0xffff
#define DVG_HIT_CHUNK 16
#define DVG_PF_SLOTS 16   // prefiltered fragments cached per sample
#define DVG_PF_BYTES 64   // bytes per cached prefiltered fragment
#define DVG_PF_CHUNK 16   // prefiltered fragments per cache chunk past the slots

// Boundary samples filed by canvas tile (edge-sampling pass), n entries
// each; tile_count / tile_start have one entry per canvas tile (+1).
struct EdgeRecords {
  float4 *a;        // boundary point (normalised canvas), normal
  float4 *b;        // local point, pdf, t
  int4 *c;          // group, shape, segment, first point
  float2 *d;        // segment t, is_stroke
  int *key, *rank, *order;
  int *tile_count, *tile_start;  // per ordering cell: [tiles * DVG_EDGE_CELLS] (+1)
  // Deferred fp64 root walks of the paired-lane pass (null job_a: none).  A
  // colour query q (= 2 * sorted sample position + side) whose queued
  // segment tests the fp32 decision leaves open hands them to the job list
  // and keeps its candidate fragments in frag; k_edge_jobs decides the jobs
  // with full warps, k_edge_finish blends the deferred queries and
  // accumulates their samples' gradients.
  int4 *job_a = nullptr;     // [job_cap] {query, result bit, shape, segment}; query -1: no job
  float4 *job_b = nullptr;   // [job_cap] {x, y, stroke radius, -} in shape space
  int4 *dq = nullptr;        // [2n] per query of a deferred sample: {first fragment (-1: finished in the
                             //   first pass), state word (dq_state), fp32 results, edge-query job bits}
  unsigned *dq_res = nullptr;  // [2n] results of the query's deferred jobs
  float4 *dq_col = nullptr;  // [2n] colour of a query finished in the first pass; of a deferred
                             //   query, the blend of the fragments its walk flushed
  int2 *frag = nullptr;      // [frag_cap] candidate fragments (key, meta) of deferred queries
  int *ds = nullptr;         // [n] sorted positions of the deferred samples
  // the root brackets of the cubic jobs (k_edge_jobs), walked one per lane by k_edge_roots
  double *job_q = nullptr;   // [5 job_cap] the job's normalised distance quintic, coefficients B..F
  int4 *task = nullptr;      // [task_cap] {job (-1: none), lower end, upper end (float bits), -}
  int *counts = nullptr;     // [8] jobs, -, fragments, deferred samples, brackets, bracket cursor, -, -
  int job_cap = 0, frag_cap = 0, task_cap = 0;
};
// Boundary samples are ordered by canvas tile and, inside a tile, by
// 2^DVG_EDGE_CELL_SHIFT-pixel square cell in Morton order.
#define DVG_EDGE_CELL_SHIFT 2
#define DVG_EDGE_CELLS ((DVG_TILE >> DVG_EDGE_CELL_SHIFT) * (DVG_TILE >> DVG_EDGE_CELL_SHIFT))

// One scene of a batched launch (dvg_batch_forward / dvg_batch_backward):
// the persistent batched kernels take an array of these in device memory
// and a work queue over the scenes' tiles or boundary samples.
struct BatchScene {
  DevScene S;
  DevRender R;
  EdgeRecords E;
  float4 *samples;  // forward sample colours
};
#define DVG_BATCH_MAX 256  // scenes per batched launch

typedef float2 v2;

#define DI __device__ __forceinline__
// out of line: large routines that would otherwise be copied into every caller
#define DN static __device__ __noinline__

DI v2 V2(float x, float y) { return make_float2(x, y); }
DI v2 add2(v2 a, v2 b) { return V2(a.x + b.x, a.y + b.y); }
DI v2 sub2(v2 a, v2 b) { return V2(a.x - b.x, a.y - b.y); }
DI v2 mul2(v2 a, v2 b) { return V2(a.x * b.x, a.y * b.y); }
DI v2 scl2(float s, v2 a) { return V2(s * a.x, s * a.y); }
DI v2 div2s(v2 a, float s) { return V2(a.x / s, a.y / s); }
DI v2 neg2(v2 a) { return V2(-a.x, -a.y); }
DI float sum2(v2 a) { return a.x + a.y; }
DI float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
DI float lensq2(v2 a) { return a.x * a.x + a.y * a.y; }
DI float len2(v2 a) { return sqrtf(lensq2(a)); }
DI float dist2(v2 a, v2 b) { return len2(sub2(b, a)); }
DI float distsq2(v2 a, v2 b) { return lensq2(sub2(b, a)); }
DI v2 normalize2(v2 a) { float l = len2(a); return V2(a.x / l, a.y / l); }
DI float4 F4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
DI float4 add4(float4 a, float4 b) { return F4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
DI float4 sub4(float4 a, float4 b) { return F4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
DI float4 scl4(float s, float4 a) { return F4(s * a.x, s * a.y, s * a.z, s * a.w); }
DI float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
DI float rmin(float a, float b) { return a < b ? a : b; }
DI float rmax(float a, float b) { return a > b ? a : b; }
DI float sq(float x) { return x * x; }
DI float clampf_(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
DI float det2(v2 a, v2 b) { return a.x * b.y - b.x * a.y; }
DI float absmax2(v2 a) { return fmaxf(fabsf(a.x), fabsf(a.y)); }

// boxes are float4 (lo.x, lo.y, hi.x, hi.y); aabb.h:15-40, 62-66
DI float4 box_empty() { return F4(INFINITY, INFINITY, -INFINITY, -INFINITY); }
DI float4 box_add(float4 b, v2 p) { return F4(rmin(p.x, b.x), rmin(p.y, b.y), rmax(p.x, b.z), rmax(p.y, b.w)); }
DI float4 box_union(float4 a, float4 b) {
  return F4(rmin(a.x, b.x), rmin(a.y, b.y), rmax(a.z, b.z), rmax(a.w, b.w));
}
DI bool box_in(float4 b, v2 p) { return p.x >= b.x && p.x <= b.z && p.y >= b.y && p.y <= b.w; }
DI bool box_in_r(float4 b, v2 p, float r) {
  return p.x >= b.x - r && p.x <= b.z + r && p.y >= b.y - r && p.y <= b.w + r;
}
// winding-ray box test (winding_number.h:33-42)
DI bool box_ray(float4 b, v2 p) {
  if (p.y < b.y || p.y > b.w) return false;
  if (p.x > b.z) return false;
  return true;
}

// 3x3 row-major transforms (matrix.h:209-229, 504-544)
DI v2 xform_pt(const float *m, v2 p) {
  float t0 = m[0] * p.x + m[1] * p.y + m[2];
  float t1 = m[3] * p.x + m[4] * p.y + m[5];
  float t2 = m[6] * p.x + m[7] * p.y + m[8];
  return V2(t0 / t2, t1 / t2);
}
DI void d_xform_pt(const float *m, v2 pt, v2 d_out, float *d_m, v2 *d_pt) {
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
DI v2 xform_normal(const float *m_inv, v2 n) {
  return normalize2(V2(m_inv[0] * n.x + m_inv[3] * n.y, m_inv[1] * n.x + m_inv[4] * n.y));
}
DI void inverse3(const float *m, float *r) {
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

// ---------------------------------------------------------------------------
// pcg32 (pcg.h:11-40): one stream per sample index, XSH-RR output.
struct Pcg { uint64_t state, inc; };
DI uint32_t pcg_next(Pcg &r) {
  uint64_t old = r.state;
  r.state = old * 6364136223846793005ULL + (r.inc | 1ULL);
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return __funnelshift_r(xs, xs, rot);
}
DI float pcg_float(Pcg &r) { return __uint_as_float((pcg_next(r) >> 9) | 0x3f800000u) - 1.0f; }
DI Pcg pcg_init(int32_t idx, uint64_t seed) {
  Pcg s;
  s.inc = (((uint64_t)(int64_t)idx + 1ULL) << 1u) | 1ULL;
  // state = 0; next(); state += K + seed; next();  (the first output is unused)
  s.state = s.inc + (0x853c49e6748fea9bULL + seed);
  s.state = s.state * 6364136223846793005ULL + s.inc;
  return s;
}

// ---------------------------------------------------------------------------
// root solvers (solve.h:5-59)
// IEEE divisions out of line for the rarely run solver paths (each inline
// division expands to ~100 instructions without fused multiply-add)
DN float fdiv(float a, float b) { return a / b; }
DN double ddiv(double a, double b) { return a / b; }
DN double dsqrt(double a) { return sqrt(a); }

DI bool solve_quadratic_f(float a, float b, float c, float *t0, float *t1) {
  float discrim = b * b - 4 * a * c;
  if (discrim < 0) return false;
  float root = sqrtf(discrim);
  float q = (b < 0) ? -0.5f * (b - root) : -0.5f * (b + root);
  *t0 = fdiv(q, a);
  *t1 = fdiv(c, q);
  if (*t0 > *t1) { float tmp = *t0; *t0 = *t1; *t1 = tmp; }
  return true;
}
DI bool solve_quadratic_d(double a, double b, double c, double *t0, double *t1) {
  double discrim = b * b - 4 * a * c;
  if (discrim < 0) return false;
  double root = dsqrt(discrim);
  double q = (b < 0) ? -0.5f * (b - root) : -0.5f * (b + root);
  *t0 = ddiv(q, a);
  *t1 = ddiv(c, q);
  if (*t0 > *t1) { double tmp = *t0; *t0 = *t1; *t1 = tmp; }
  return true;
}
// solve_cubic<double> (solve.h:24-58).  The three trigonometric roots share
// one cos call (theta + 0 = theta for theta = acos(.) >= 0), and the one-root
// branch's two pow calls one (R + s for R > 0, -R + s otherwise, is |R| + s).
DN int solve_cubic_d(double a, double b, double c, double d, double t[3]) {
  if (fabs(a) < 1e-6f) return solve_quadratic_d(b, c, d, &t[0], &t[1]) ? 2 : 0;
  b = ddiv(b, a); c = ddiv(c, a); d = ddiv(d, a);
  double Q = ddiv(b * b - 3 * c, 9.f);
  double R = ddiv(2 * b * b * b - 9 * b * c + 27 * d, 54.f);
  if (R * R < Q * Q * Q) {
    double theta = acos(ddiv(R, dsqrt(Q * Q * Q)));
    double sQ = dsqrt(Q);
    double b3 = ddiv(b, 3.f);
    const double off[3] = {0.0, 2.f * DVG_PI, -(2.f * DVG_PI)};
    #pragma unroll 1
    for (int k = 0; k < 3; k++) t[k] = -2.f * sQ * cos(ddiv(theta + off[k], 3.f)) - b3;
    return 3;
  } else {
    double pw = pow(fabs(R) + dsqrt(R * R - Q * Q * Q), (double)(1. / 3.));
    double A = R > 0 ? -pw : pw;
    double B = fabs(A) > 1e-6f ? ddiv(Q, A) : 0.0;
    t[0] = (A + B) - ddiv(b, 3.0);
    return 1;
  }
}
// solve_cubic<float>: the reference's unqualified sqrt/acos/cos/pow bind to
// the double-precision functions, so intermediates are double until stored
// back into a float.
DN int solve_cubic_f(float a, float b, float c, float d, float t[3]) {
  if (fabsf(a) < 1e-6f) return solve_quadratic_f(b, c, d, &t[0], &t[1]) ? 2 : 0;
  b = fdiv(b, a); c = fdiv(c, a); d = fdiv(d, a);
  float Q = fdiv(b * b - 3 * c, 9.f);
  float R = fdiv(2 * b * b * b - 9 * b * c + 27 * d, 54.f);
  if (R * R < Q * Q * Q) {
    float theta = (float)acos(ddiv((double)R, dsqrt((double)(Q * Q * Q))));
    double sQ = dsqrt((double)Q);
    double b3 = (double)fdiv(b, 3.f);
    const float off[3] = {0.f, 2.f * (float)DVG_PI, -(2.f * (float)DVG_PI)};
    #pragma unroll 1
    for (int k = 0; k < 3; k++) t[k] = (float)(-2.f * sQ * cos((double)fdiv(theta + off[k], 3.f)) - b3);
    return 3;
  } else {
    double third = (double)(float)(1. / 3.);
    double pw = pow((double)fabsf(R) + dsqrt((double)(R * R - Q * Q * Q)), third);
    float A = R > 0 ? (float)(-pw) : (float)pw;
    float B = fabsf(A) > 1e-6f ? fdiv(Q, A) : 0.f;
    t[0] = (A + B) - fdiv(b, 3.f);
    return 1;
  }
}

// ---------------------------------------------------------------------------
// pixel filters (filter.h:22-106).  DVG_GAUSSIAN has no counterpart in the
// reference: a separable Gaussian of standard deviation r / 2 shifted down
// to reach 0 at the edge of the support |dx|, |dy| <= r (continuous there,
// so its radius gradient needs no boundary term):
//   w = g(dx) g(dy),  g(x) = exp(-2 x^2 / r^2) - exp(-2).
// Weights need no normalisation: pixels divide by their weight sums.
DI float gauss_1d(float x, float r) { return expf(-2.f * sq(x) / sq(r)) - expf(-2.f); }
DI float filter_weight(int type, float r, float dx, float dy) {
  if (fabsf(dx) > r || fabsf(dy) > r) return 0;
  if (type == DVG_GAUSSIAN) return r > 0.f ? gauss_1d(dx, r) * gauss_1d(dy, r) : 0.f;
  if (type == DVG_BOX) return 1.f / sq(2 * r);
  if (type == DVG_TENT) return (r - fabsf(dx)) * (r - fabsf(dy)) / sq(sq(r));
  if (type == DVG_PARABOLIC) return (4.f / 3.f) * (1 - sq(dx / r)) * (4.f / 3.f) * (1 - sq(dy / r));
  float ndx = (dx / (2 * r)) + 0.5f, ndy = (dy / (2 * r)) + 0.5f;
  return 0.5f * (1.f - cosf((float)(2 * DVG_PI) * ndx)) * 0.5f * (1.f - cosf((float)(2 * DVG_PI) * ndy)) / sq(r);
}
DI float d_filter_weight(int type, float r, float dx, float dy, float d_ret) {
  if (type == DVG_GAUSSIAN) {
    if (!(r > 0.f) || fabsf(dx) > r || fabsf(dy) > r) return 0.f;
    float r3 = r * r * r;  // dg/dr = exp(-2 x^2 / r^2) 4 x^2 / r^3
    float dgx = expf(-2.f * sq(dx) / sq(r)) * 4.f * sq(dx) / r3, dgy = expf(-2.f * sq(dy) / sq(r)) * 4.f * sq(dy) / r3;
    return d_ret * (dgx * gauss_1d(dy, r) + gauss_1d(dx, r) * dgy);
  }
  if (type == DVG_BOX) {
    return d_ret * (-2) * 2 * r / ((2 * r) * (2 * r) * (2 * r));
  } else if (type == DVG_TENT) {
    float fx = r - fabsf(dx), fy = r - fabsf(dy);
    float norm = 1 / sq(r);
    float d_fx = d_ret * fy * norm, d_fy = d_ret * fx * norm, d_norm = d_ret * fx * fy;
    return d_fx + d_fy + (-4) * d_norm / (float)pow((double)r, 5.0);
  } else if (type == DVG_PARABOLIC) {
    float r3 = r * r * r;
    return -(2 * sq(dx) + 2 * sq(dy)) / r3;
  } else {
    float ndx = (dx / (2 * r)) + 0.5f, ndy = (dy / (2 * r)) + 0.5f;
    float fx = 0.5f * (1.f - cosf((float)(2 * DVG_PI) * ndx));
    float fy = 0.5f * (1.f - cosf((float)(2 * DVG_PI) * ndy));
    float norm = 1 / sq(r);
    float d_fx = d_ret * fy * norm, d_fy = d_ret * fx * norm, d_norm = d_ret * fx * fy;
    float d_ndx = d_fx * 0.5f * sinf((float)(2 * DVG_PI) * ndx) * (float)(2 * DVG_PI);
    float d_ndy = d_fy * 0.5f * sinf((float)(2 * DVG_PI) * ndy) * (float)(2 * DVG_PI);
    return d_ndx * (-2 * dx / sq(2 * r)) + d_ndy * (-2 * dy / sq(2 * r)) + (-2) * d_norm / (r * r * r);
  }
}

// ---------------------------------------------------------------------------
// scene accessors
#define SI(S, s, f) __ldg(&(S).shape_info[(s) * DVG_SHAPE_INFO_STRIDE + (f)])
#define GI(S, g, f) __ldg(&(S).group_info[(g) * DVG_GROUP_INFO_STRIDE + (f)])

DI v2 path_pt(const DevScene &S, int po, int i) {
  return V2(__ldg(&S.P[po + 2 * i]), __ldg(&S.P[po + 2 * i + 1]));
}
DI float pget(const DevScene &S, int off) { return __ldg(&S.P[off]); }
DI float stroke_width(const DevScene &S, int s) { return pget(S, SI(S, s, DVG_SHAPE_STROKE_WIDTH_OFF)); }
DI void flag_error(const DevScene &S, unsigned bit) { atomicOr(S.err, bit); }

DI v2 eval_quad(v2 p0, v2 p1, v2 p2, float t) {
  float tt = 1 - t;
  return add2(add2(scl2(tt * tt, p0), scl2(2 * tt * t, p1)), scl2(t * t, p2));
}
DI v2 eval_cubic(v2 p0, v2 p1, v2 p2, v2 p3, float t) {
  float tt = 1 - t;
  return add2(add2(add2(scl2(tt * tt * tt, p0), scl2(3 * tt * tt * t, p1)), scl2(3 * tt * t * t, p2)),
              scl2(t * t * t, p3));
}

// log2 of the stroke records per tile-mask bit of a group with n records:
// one record per bit up to 32 records, else the fewest records per bit (a
// power of two) that fit the group in 32 bits
DI int rec_chunk_shift(int n) {
  int c = 0;
  while ((n + (1 << c) - 1) >> c > 32) c++;
  return c;
}

// Candidate groups for a canvas-space point: the point's tile list, or all
// groups outside the tile grid.  Returns true when the tile list is used.
DI bool cand_range(const DevScene &S, v2 pt, int &begin, int &end) {
  float fx = floorf(pt.x / DVG_TILE), fy = floorf(pt.y / DVG_TILE);
  if (fx >= 0 && fy >= 0 && fx < S.tiles_x && fy < S.tiles_y) {
    int t = (int)fy * S.tiles_x + (int)fx;
    begin = __ldg(&S.tile_start[t]);
    end = __ldg(&S.tile_start[t + 1]);
    return true;
  }
  begin = 0;
  end = S.num_groups;
  return false;
}

// ---------------------------------------------------------------------------
// winding numbers (winding_number.h:9-202)

// Certified fp32 winding contribution of one cubic segment for the +x ray
// from pt.  y(t) is split at its extrema into monotone pieces; a piece whose
// end values straddle pt.y holds exactly one simple crossing, found by
// bisection, and counts +-1 when the crossing lies right of pt.  Every
// decision (end values against pt.y, crossing x against pt.x) must clear a
// rounding margin; otherwise DVG_WINDING_UNDECIDED is returned and the caller
// runs the reference's fp64 cubic solve.  With every decision clear of the
// margin the reference's closed-form roots are simple roots at the same
// crossings, so both count the same.  When the control points all lie right
// of pt by more than the crossing margin, so does every crossing (the curve
// stays in their convex hull), and the pieces are counted without bisection.
#define DVG_WINDING_UNDECIDED (-1000)
DI float cubic_y(float a, float b, float c, float d, float t) { return ((a * t + b) * t + c) * t + d; }
DI int winding_cubic_fast(v2 p0, v2 p1, v2 p2, v2 p3, v2 pt) {
  float m = 2e-5f * fmaxf(fmaxf(absmax2(p0), absmax2(p1)), fmaxf(fmaxf(absmax2(p2), absmax2(p3)), absmax2(pt))) + 1e-4f;
  float ay = -p0.y + 3 * p1.y - 3 * p2.y + p3.y, by = 3 * p0.y - 6 * p1.y + 3 * p2.y, cy = -3 * p0.y + 3 * p1.y,
        dy = p0.y - pt.y;
  float ax = -p0.x + 3 * p1.x - 3 * p2.x + p3.x, bx = 3 * p0.x - 6 * p1.x + 3 * p2.x, cx = -3 * p0.x + 3 * p1.x,
        dx = p0.x - pt.x;
  // split points: roots of y'(t) = 3 ay t^2 + 2 by t + cy inside (0, 1)
  float ts[4];
  int nt = 0;
  ts[nt++] = 0.f;
  {
    float qa = 3 * ay, qb = 2 * by, qc = cy;
    float e0 = -1.f, e1 = -1.f;
    if (fabsf(qa) > 1e-12f) {
      float disc = qb * qb - 4 * qa * qc;
      if (disc >= 0.f) {
        float sq_ = sqrtf(disc);
        float q = qb < 0 ? -0.5f * (qb - sq_) : -0.5f * (qb + sq_);
        e0 = q / qa;
        e1 = q != 0.f ? qc / q : -1.f;
      }
    } else if (fabsf(qb) > 1e-12f) {
      e0 = -qc / qb;
    }
    if (e0 > e1) { float tmp = e0; e0 = e1; e1 = tmp; }
    if (e0 > 0.f && e0 < 1.f) ts[nt++] = e0;
    if (e1 > 0.f && e1 < 1.f && e1 != e0) ts[nt++] = e1;
  }
  ts[nt++] = 1.f;
  float span = fmaxf(fmaxf(fabsf(ax), fabsf(bx)), fmaxf(fabsf(cx), 1.f));
  float xmargin = 4.f * m + 1e-6f * span;
  bool right = fminf(fminf(p0.x, p1.x), fminf(p2.x, p3.x)) - pt.x > xmargin;
  int w = 0;
  float ya = cubic_y(ay, by, cy, dy, ts[0]);
  if (fabsf(ya) <= m) return DVG_WINDING_UNDECIDED;
  #pragma unroll 1
  for (int k = 1; k < nt; k++) {
    float yb = cubic_y(ay, by, cy, dy, ts[k]);
    if (fabsf(yb) <= m) return DVG_WINDING_UNDECIDED;
    if ((ya < 0.f) != (yb < 0.f) && right) {
      w += yb > ya ? 1 : -1;
    } else if ((ya < 0.f) != (yb < 0.f)) {
      float lo = ts[k - 1], hi = ts[k];
      bool up = yb > ya;
      #pragma unroll 1
      for (int it = 0; it < 26; it++) {
        float mid = 0.5f * (lo + hi);
        float ym = cubic_y(ay, by, cy, dy, mid);
        if ((ym > 0.f) == up) hi = mid; else lo = mid;
      }
      float xs = cubic_y(ax, bx, cx, dx, 0.5f * (lo + hi));
      if (fabsf(xs) <= xmargin) return DVG_WINDING_UNDECIDED;
      if (xs > 0.f) w += up ? 1 : -1;
    }
    ya = yb;
  }
  return w;
}

DI int winding_segment(const DevScene &S, int po, int np, int nc, int i0, v2 pt) {
  int w = 0;
  if (nc == 0) {
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, (i0 + 1) % np);
    if (p1.y != p0.y) {
      float t = (pt.y - p0.y) / (p1.y - p0.y);
      if (t >= 0 && t <= 1) {
        float tp = p0.x - pt.x + t * (p1.x - p0.x);
        if (tp >= 0) w += (p1.y - p0.y > 0) ? 1 : -1;
      }
    }
  } else if (nc == 1) {
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1), p2 = path_pt(S, po, (i0 + 2) % np);
    float t[2];
    if (solve_quadratic_f(p0.y - 2 * p1.y + p2.y, -2 * p0.y + 2 * p1.y, p0.y - pt.y, &t[0], &t[1])) {
      for (int j = 0; j < 2; j++) {
        if (t[j] >= 0 && t[j] <= 1) {
          float tp = (p0.x - 2 * p1.x + p2.x) * t[j] * t[j] + (-2 * p0.x + 2 * p1.x) * t[j] + p0.x - pt.x;
          if (tp >= 0) w += (2 * (p0.y - 2 * p1.y + p2.y) * t[j] + (-2 * p0.y + 2 * p1.y) > 0) ? 1 : -1;
        }
      }
    }
  } else {
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1), p2 = path_pt(S, po, i0 + 2),
       p3 = path_pt(S, po, (i0 + 3) % np);
    int fw = winding_cubic_fast(p0, p1, p2, p3, pt);
    if (fw != DVG_WINDING_UNDECIDED) return fw;
    double t[3];
    int n = solve_cubic_d((double)(-p0.y + 3 * p1.y - 3 * p2.y + p3.y), (double)(3 * p0.y - 6 * p1.y + 3 * p2.y),
                          (double)(-3 * p0.y + 3 * p1.y), (double)(p0.y - pt.y), t);
    for (int j = 0; j < n; j++) {
      if (t[j] >= 0 && t[j] <= 1) {
        double tp = (-p0.x + 3 * p1.x - 3 * p2.x + p3.x) * t[j] * t[j] * t[j] +
                    (3 * p0.x - 6 * p1.x + 3 * p2.x) * t[j] * t[j] + (-3 * p0.x + 3 * p1.x) * t[j] + p0.x - pt.x;
        if (tp > 0) {
          w += (3 * (-p0.y + 3 * p1.y - 3 * p2.y + p3.y) * t[j] * t[j] +
                    2 * (3 * p0.y - 6 * p1.y + 3 * p2.y) * t[j] + (-3 * p0.y + 3 * p1.y) > 0)
                   ? 1 : -1;
        }
      }
    }
  }
  return w;
}

// Band of y in path s's band lists: monotone in y and clamped to the bands,
// so a segment whose box spans [ylo, yhi] is listed in every band that
// band_of maps a y of [ylo, yhi] to.
DI int band_of(float2 geo, int nb, float y) {
  float f = (y - geo.x) * geo.y;
  f = fminf(fmaxf(f, 0.f), (float)(nb - 1));
  return (int)f;
}

// The band lists of path s that hold every segment whose box can meet the
// y-range [ylo, yhi]: returns false (scan all segments) unless the path has
// band lists this call and the range falls in at most two bands; else
// [b0, e0) and [b1, e1) are entries of S.band_seg (the second range empty
// for one band), each in ascending visiting rank.  Lists skip only segments
// that the callers' own box tests would skip, so results do not change.
DI bool band_lists(const DevScene &S, int s, float ylo, float yhi, int &b0, int &e0, int &b1, int &e1) {
  if (!S.band_n) return false;
  int nb = __ldg(&S.band_n[s]);
  if (nb <= 0 || !(ylo == ylo) || !(yhi == yhi)) return false;
  float2 geo = __ldg(&S.band_geo[s]);
  int lo = band_of(geo, nb, ylo), hi = band_of(geo, nb, yhi);
  if (hi > lo + 1) return false;
  int4 sb = __ldg(&S.shape_band[s]);
  const int *st = S.band_start + sb.y;
  b0 = sb.z + __ldg(&st[lo]);
  e0 = sb.z + __ldg(&st[lo + 1]);
  b1 = e1 = e0;
  if (hi > lo) {
    b1 = e0;
    e1 = sb.z + __ldg(&st[hi + 1]);
  }
  return true;
}

// Next visiting rank of the merge of two rank-sorted band lists (a segment
// in both bands comes once); -1 when both are exhausted.
DI int band_next(const DevScene &S, int &i, int e0, int &j, int e1) {
  int a = i < e0 ? __ldg(&S.band_seg[i]) : 0x7fffffff, b = j < e1 ? __ldg(&S.band_seg[j]) : 0x7fffffff;
  if (a == 0x7fffffff && b == 0x7fffffff) return -1;
  if (a <= b) i++;
  if (b <= a) j++;
  return a < b ? a : b;
}

// Winding number of a path with band lists: only the segments of pt's band
// (band_lists; the same crossings as winding_shape's full scan).
DN int winding_banded(const DevScene &S, int s, int po, int np, int so, v2 pt) {
  int w = 0, b, e, b1, e1;
  if (band_lists(S, s, pt.y, pt.y, b, e, b1, e1)) {
    #pragma unroll 1
    for (int k = b; k < e; k++) {
      int i = __ldg(&S.seg_order[so + __ldg(&S.band_seg[k])]);
      if (!box_ray(S.seg_box[so + i], pt)) continue;
      w += winding_segment(S, po, np, __ldg(&S.segment_ctrl[so + i]), __ldg(&S.seg_point[so + i]), pt);
    }
    return w;
  }
  int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS);  // NaN point: every segment, as the full scan
  #pragma unroll 1
  for (int i = 0; i < nseg; i++) {
    if (!box_ray(S.seg_box[so + i], pt)) continue;
    w += winding_segment(S, po, np, __ldg(&S.segment_ctrl[so + i]), __ldg(&S.seg_point[so + i]), pt);
  }
  return w;
}

// Winding number of shape s at pt; with BANDED (the scene has band lists),
// paths that have band lists scan only pt's band.
template <bool BANDED>
DI int winding_shape(const DevScene &S, int s, v2 pt) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    v2 c = V2(pget(S, po + 1), pget(S, po + 2));
    float r = pget(S, po);
    return distsq2(c, pt) < r * r ? 1 : 0;
  } else if (kind == DVG_ELLIPSE) {
    v2 r = V2(pget(S, po), pget(S, po + 1)), c = V2(pget(S, po + 2), pget(S, po + 3));
    return (sq(c.x - pt.x) / sq(r.x) + sq(c.y - pt.y) / sq(r.y) < 1) ? 1 : 0;
  } else if (kind == DVG_RECT) {
    return (pt.x > pget(S, po) && pt.x < pget(S, po + 2) && pt.y > pget(S, po + 1) && pt.y < pget(S, po + 3)) ? 1 : 0;
  }
  int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
  if (BANDED && __ldg(&S.band_n[s]) > 0) return winding_banded(S, s, po, np, so, pt);
  int w = 0;
  #pragma unroll 1
  for (int i = 0; i < nseg; i++) {
    if (nseg > 1 && !box_ray(S.seg_box[so + i], pt)) continue;
    w += winding_segment(S, po, np, __ldg(&S.segment_ctrl[so + i]), __ldg(&S.seg_point[so + i]), pt);
  }
  return w;
}

struct EdgeQ { int group, shape, hit; };

// is_inside (diffvg.cpp:33-87).  Scenes with band lists take the
// BANDED instance (one test at entry, so the common instance is unchanged).
template <bool BANDED>
DI bool group_inside_body(const DevScene &S, int g, v2 pt, EdgeQ *eq) {
  v2 lp = xform_pt(S.c2s + 9 * g, pt);
  if (!box_in(S.g_local_box[g], lp)) return false;
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  int eo = GI(S, g, DVG_GROUP_EVEN_ODD);
  int w = 0;
  #pragma unroll 1
  for (int k = 0; k < nsh; k++) {
    int s = __ldg(&S.group_shapes[off + k]);
    if (nsh > 1 && !box_in(S.s_box[s], lp)) continue;
    int ws = winding_shape<BANDED>(S, s, lp);
    w += ws;
    if (eq && eq->group == g && eq->shape == s) {
      if ((eo && abs(ws) % 2 == 1) || (!eo && ws != 0)) eq->hit = 1;
    }
  }
  return eo ? (abs(w) % 2 == 1) : (w != 0);
}
DN bool group_inside_banded(const DevScene &S, int g, v2 pt, EdgeQ *eq) { return group_inside_body<true>(S, g, pt, eq); }
DN bool group_inside(const DevScene &S, int g, v2 pt, EdgeQ *eq) {
  if (S.band_n) return group_inside_banded(S, g, pt, eq);
  return group_inside_body<false>(S, g, pt, eq);
}

// ---------------------------------------------------------------------------
// stroke coverage (within_distance.h:8-446)

// quadratic_closest_pt_approx (vector.h:787-817)
DN v2 quad_closest_approx(v2 b0, v2 b1, v2 b2, v2 pt, float *t_out) {
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

// distance quintic of a cubic segment (within_distance.h:150-167), normalised
struct Quintic { double A, B, C, D, E, F; };
DI Quintic cubic_quintic(v2 p0, v2 p1, v2 p2, v2 p3, v2 pt) {
  v2 a = add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3);
  v2 b = add2(sub2(scl2(3, p0), scl2(6, p1)), scl2(3, p2));
  v2 c = add2(scl2(-3, p0), scl2(3, p1));
  v2 e = sub2(p0, pt);
  Quintic q;
  q.A = (double)(3 * sum2(mul2(a, a)));
  q.B = (double)(5 * sum2(mul2(a, b)));
  q.C = (double)(4 * sum2(mul2(a, c)) + 2 * sum2(mul2(b, b)));
  q.D = (double)(3 * (sum2(mul2(b, c)) + sum2(mul2(a, e))));
  q.E = (double)(sum2(mul2(c, c)) + 2 * sum2(mul2(e, b)));
  q.F = (double)(sum2(mul2(e, c)));
  q.B = ddiv(q.B, q.A); q.C = ddiv(q.C, q.A); q.D = ddiv(q.D, q.A); q.E = ddiv(q.E, q.A); q.F = ddiv(q.F, q.A);
  return q;
}
DI double quintic_eval(const Quintic &q, double t) {
  return t * t * t * t * t + q.B * t * t * t * t + q.C * t * t * t + q.D * t * t + q.E * t + q.F;
}
DI double quintic_deriv(const Quintic &q, double t) {
  return 5 * t * t * t * t + 4 * q.B * t * t * t + 3 * q.C * t * t + 2 * q.D * t + q.E;
}
// isolator intervals (within_distance.h:181-236); a slot that the reference
// leaves uninitialised when -B/5 is outside [0,1] holds -1 (skipped).
DI int quintic_intervals(const Quintic &q, float iv[4]) {
  double p1A = (2 / 5.f) * q.C - (4 / 25.f) * q.B * q.B;
  double p1B = (3 / 5.f) * q.D - (3 / 25.f) * q.B * q.C;
  double p1C = (4 / 5.f) * q.E - (2 / 25.f) * q.B * q.D;
  double p1D = q.F - ddiv(q.B * q.E, 25.f);
  double q_root = ddiv(-q.B, 5.f);
  double pr[3];
  int ns = solve_cubic_d(p1A, p1B, p1C, p1D, pr);
  iv[0] = (q_root >= 0 && q_root <= 1) ? (float)q_root : -1.0f;
  for (int j = 0; j < ns; j++) iv[j + 1] = (float)pr[j];
  int n = 1 + ns;
  for (int j = 1; j < n; j++)
    for (int k = j; k > 0 && iv[k - 1] > iv[k]; k--) { float tmp = iv[k]; iv[k] = iv[k - 1]; iv[k - 1] = tmp; }
  return n;
}
// safeguarded Newton / bisection in one bracket (within_distance.h:251-269).
// When the caller swapped the bracket ends (q decreasing), lb > ub holds for
// the whole loop, the test t in [lb, ub] always fails and every iteration
// restarts from the midpoint: the reference's Newton update is dead work
// there and is skipped, which leaves every result unchanged.
DI float quintic_root(const Quintic &q, float lb, float ub) {
  float t = 0.5f * (lb + ub);
  #pragma unroll 1
  for (int it = 0; it < 20; it++) {
    if (!(t >= lb && t <= ub)) t = 0.5f * (lb + ub);
    double value = quintic_eval(q, t);
    if (fabs(value) < 1e-5f || it == 19) break;
    if (value > 0.f) ub = t; else lb = t;
    if (lb > ub) continue;  // the next iteration restarts from the midpoint
    double derivative = quintic_deriv(q, t);
    t = (float)(t - ddiv(value, derivative));
  }
  return t;
}

// quintic value at a bracket end; consecutive brackets share an end, so the
// previous value is reused (same argument, same result)
DI double quintic_eval_cached(const Quintic &q, float t, float &ct, double &cv) {
  if (t == ct) return cv;
  ct = t;
  cv = quintic_eval(q, t);
  return cv;
}

// ---------------------------------------------------------------------------
// Conservative fp32 distance bounds that skip fp64 root solves whose outcome
// is already decided.  A Bezier curve lies in the convex hull of its control
// points, and the hull lies in the capsule of radius max_i dist(p_i, chord)
// around the chord p0-pn, so
//     dist(pt, curve) >= dist(pt, chord) - max_i dist(p_i, chord).
// Splitting at t = 1/2 (de Casteljau) shrinks the capsule radius 4x per
// level; curve_stroke_fast walks the subdivision tree.  far_margin() covers
// the fp32 rounding of the bound and of the reference's own fp32 distance
// evaluation, so a segment reported far is one on which the reference's test
// fails as well (the stroke test and the closest-point search use it alike).
DI float dist_to_seg(v2 a, v2 b, v2 p) {
  v2 ab = sub2(b, a);
  float l2 = dot2(ab, ab);
  float t = l2 > 0.f ? clampf_(dot2(sub2(p, a), ab) / l2, 0.f, 1.f) : 0.f;
  return len2(sub2(add2(a, scl2(t, ab)), p));
}
DI float far_margin(float m) { return 1e-5f * m + 1e-4f; }
#define DVG_SUBDIV_DEPTH 8
DI v2 lerp2(v2 a, v2 b, float u) { return V2(a.x + u * (b.x - a.x), a.y + u * (b.y - a.y)); }
DI v2 cubic_blossom(v2 p0, v2 p1, v2 p2, v2 p3, float u, float v, float w) {
  v2 a0 = lerp2(p0, p1, u), a1 = lerp2(p1, p2, u), a2 = lerp2(p2, p3, u);
  v2 b0 = lerp2(a0, a1, v), b1 = lerp2(a1, a2, v);
  return lerp2(b0, b1, w);
}
DI v2 quad_blossom(v2 p0, v2 p1, v2 p2, float u, float v) {
  return lerp2(lerp2(p0, p1, u), lerp2(p1, p2, u), v);
}
// Levels 0..DVG_TREE_DEPTH of each curved segment's subdivision tree are
// tabulated per call (k_seg_tree): the curve points at t = k / 2^D (the end
// points of every tabulated piece) and each piece's hull width, the largest
// distance of its inner control points from its chord.  Deeper pieces are
// formed from blossoms on the fly.  Tabulated and on-the-fly pieces hold the
// same fp32 values.
#define DVG_TREE_DEPTH 5
#define DVG_TREE_PTS ((1 << DVG_TREE_DEPTH) + 1)
#define DVG_TREE_NODES (2 << DVG_TREE_DEPTH)  // heap order, entry 0 unused

// distance from p to the segment ab greater than T (T >= 0), without roots or divisions
DI bool seg_far(v2 a, v2 b, v2 p, float T) {
  v2 ab = sub2(b, a), ap = sub2(p, a);
  float T2 = T * T;
  float dt = dot2(ap, ab);
  if (dt <= 0.f) return dot2(ap, ap) > T2;
  float l2 = dot2(ab, ab);
  if (dt >= l2) {
    v2 bp = sub2(p, b);
    return dot2(bp, bp) > T2;
  }
  float cr = ap.x * ab.y - ap.y * ab.x;
  return cr * cr > T2 * l2;
}
DI float cubic_hull_width(v2 q0, v2 q1, v2 q2, v2 q3) { return fmaxf(dist_to_seg(q0, q3, q1), dist_to_seg(q0, q3, q2)); }
DI float quad_hull_width(v2 q0, v2 q1, v2 q2) { return dist_to_seg(q0, q2, q1); }

// Certified fp32 outside proof for the stroke test of one Bezier segment
// (nc = 1 quadratic: p3 unused; nc = 2 cubic).  The segment is subdivided
// (stackless depth-first walk of the binary subdivision tree) and a piece
// whose capsule bound (distance to its chord less its hull width) is farther
// than r_out + m is pruned.  tp / th: the segment's tabulated tree, or null.
// Returns 0 when every piece is pruned: no point of the curve is within the
// stroke radius, so the reference's candidates (end points and quintic or
// cubic roots, all on the curve) fail its test as well.  Returns -2
// otherwise, early when a curve point is closer than r_out - m, and the
// caller runs the root-walk decision.  No inside proof is attempted: the
// reference's quintic root isolation can miss the closest root (two roots in
// one isolation interval) and then reports "outside" for a sample that is
// geometrically inside; the renderer reproduces the reference.
template <int NC>
DN int curve_stroke_fast(v2 p0, v2 p1, v2 p2, v2 p3, const float2 *tp, const float *th, v2 pt, float r_out,
                         float m) {
  float thr_out = r_out + m;
  float near = r_out - m;
  float near2 = near > 0.f ? near * near : -1.f;
  unsigned node = 1;
  #pragma unroll 1
  for (int guard = 0; guard < (2 << DVG_SUBDIV_DEPTH) + 2; guard++) {
    int d = 31 - __clz(node);
    v2 q0, qe;
    float h;
    if (tp && d <= DVG_TREE_DEPTH) {
      unsigned k = node - (1u << d);
      int sh = DVG_TREE_DEPTH - d;
      q0 = tp[k << sh];
      qe = tp[(k + 1) << sh];
      h = th[node];
    } else {
      float scale = __int_as_float((127 - d) << 23);  // 2^-d, exact
      float ta = (float)(node - (1u << d)) * scale, tb = ta + scale;
      if (NC == 2) {
        q0 = cubic_blossom(p0, p1, p2, p3, ta, ta, ta);
        qe = cubic_blossom(p0, p1, p2, p3, tb, tb, tb);
        h = cubic_hull_width(q0, cubic_blossom(p0, p1, p2, p3, ta, ta, tb), cubic_blossom(p0, p1, p2, p3, ta, tb, tb),
                             qe);
      } else {
        q0 = quad_blossom(p0, p1, p2, ta, ta);
        qe = quad_blossom(p0, p1, p2, tb, tb);
        h = quad_hull_width(q0, quad_blossom(p0, p1, p2, ta, tb), qe);
      }
    }
    // a curve point this close: no outside proof can exist
    if (distsq2(q0, pt) < near2 || distsq2(qe, pt) < near2) return -2;
    if (!seg_far(q0, qe, pt, thr_out + h)) {
      if (d >= DVG_SUBDIV_DEPTH) return -2;
      node <<= 1;
      continue;
    }
    while (node & 1u) node >>= 1;
    if (node == 0u) return 0;
    node += 1;
  }
  return -2;
}

// ---------------------------------------------------------------------------
// fp32 decision of the reference's cubic-segment stroke test.
//
// The reference decides a point against a cubic segment by isolating the
// roots of the normalised distance quintic Q (breakpoints: -B/5 and the roots
// of the isolator cubic Q - (t/5 + B/25) Q', within_distance.h:181-236),
// walking the brackets whose ends change sign (the lower end stays put
// through brackets without a sign change, within_distance.h:237-240), running
// a safeguarded Newton iteration in each that stops where |Q| < 1e-5 or after
// 20 steps (within_distance.h:244-261), and testing the distance at the
// stopping point against the interpolated radius.  All of it runs in fp64
// there.  cubic_stroke_decide repeats the same structure in fp32 with error
// enclosures: every breakpoint carries a certified radius, every sign the
// reference reads must be certain, each sign-change bracket must hold one
// simple root (Bernstein bounds of Q' on subdivided pieces) and no other
// place where the Newton iteration could stop, and the distance at the root
// must clear the radius by a margin that covers where in the stopping window
// the reference lands.  Returns 1 or 0 when that decides the outcome, 2 when
// any enclosure is inconclusive (the fp64 solve then runs).
#define DVG_EMU_NEWTON 6  // Newton steps per root (each root is certified afterwards)
DI float emu_p3(float c3, float c2, float c1, float c0, float t) { return ((c3 * t + c2) * t + c1) * t + c0; }
DI float emu_q(const float n[6], float t) { return ((((t + n[1]) * t + n[2]) * t + n[3]) * t + n[4]) * t + n[5]; }
// Bernstein coefficients on [l,u] of the quartic with [0,1]-Bernstein coefficients b (blossoming)
DI void emu_blossom4(const float b[5], float l, float u, float c[5]) {
#pragma unroll
  for (int k = 0; k < 5; k++) {
    float w[5];
#pragma unroll
    for (int i = 0; i < 5; i++) w[i] = b[i];
#pragma unroll
    for (int lev = 0; lev < 4; lev++) {
      float t = lev < 4 - k ? l : u;
#pragma unroll
      for (int i = 0; i < 4 - lev; i++) w[i] = w[i] + t * (w[i + 1] - w[i]);
    }
    c[k] = w[0];
  }
}
// roots in (0,1) of c3 t^3 + c2 t^2 + c1 t + c0, one slot per monotone piece
// (split at the stationary points), each with a certified enclosure radius
// (the sign change at root +- rad is certain); false when a stationary
// point or an end sits within del of zero, or an enclosure fails
DI bool emu_cubic_roots3(float c3, float c2, float c1, float c0, float del, float root[3], float rad[3], bool has[3]) {
  // stationary points (their rounding is covered by the end checks below: a
  // piece's end within del of zero makes the result uncertain)
  float qa = 3 * c3, qb = 2 * c2, qc = c1, e0 = -1.f, e1 = -1.f;
  float sc = fabsf(qa) + fabsf(qb) + fabsf(qc);
  if (fabsf(qa) > 1e-7f * sc) {
    float disc = qb * qb - 4 * qa * qc;
    if (disc >= 0.f) {
      float s = sqrtf(disc);
      float q = qb < 0 ? -0.5f * (qb - s) : -0.5f * (qb + s);
      e0 = __fdividef(q, qa);
      e1 = q != 0.f ? __fdividef(qc, q) : -1.f;
    }
  } else if (fabsf(qb) > 1e-7f * sc) {
    e0 = __fdividef(-qc, qb);
  }
  if (e0 > e1) { float tmp = e0; e0 = e1; e1 = tmp; }
  bool h0 = e0 > 0.f && e0 < 1.f, h1 = e1 > 0.f && e1 < 1.f && e1 != e0;
  float t1 = h0 ? e0 : (h1 ? e1 : 1.f), t2 = (h0 && h1) ? e1 : 1.f;
  float rr[3] = {0.f, 0.f, 0.f}, ee[3] = {0.f, 0.f, 0.f};
  bool hh[3] = {false, false, false};
  bool ok = true;
  float ta = 0.f, ya = emu_p3(c3, c2, c1, c0, 0.f);
  ok = ok && fabsf(ya) > del;
  #pragma unroll 1
  for (int k = 1; k < 4; k++) {  // the monotone pieces [0,t1], [t1,t2], [t2,1]
    float tb = k == 1 ? t1 : (k == 2 ? t2 : 1.f);
    float yb = emu_p3(c3, c2, c1, c0, tb);
    ok = ok && fabsf(yb) > del;
    if (ok && (ya < 0) != (yb < 0)) {
      float lo = ta, hi = tb;
      bool up = yb > ya;
      float r = 0.5f * (lo + hi);
      #pragma unroll 1
      for (int it = 0; it < DVG_EMU_NEWTON; it++) {  // Newton kept inside the bracket
        float y = emu_p3(c3, c2, c1, c0, r), dy = (3 * c3 * r + 2 * c2) * r + c1;
        if ((y > 0) == up) hi = r; else lo = r;
        float nr = r - __fdividef(y, dy);
        r = (nr >= lo && nr <= hi) ? nr : 0.5f * (lo + hi);
      }
      float dp = fabsf((3 * c3 * r + 2 * c2) * r + c1);
      float eps = fmaxf(4e-7f, __fdividef(4.f * del, dp));
      float ym = emu_p3(c3, c2, c1, c0, r - eps), yp = emu_p3(c3, c2, c1, c0, r + eps);
      ok = ok && dp > 0.f && fabsf(ym) > del && fabsf(yp) > del && ((ym < 0) != (yp < 0));
      // slot k - 1, kept in registers
      rr[0] = k == 1 ? r : rr[0]; rr[1] = k == 2 ? r : rr[1]; rr[2] = k == 3 ? r : rr[2];
      ee[0] = k == 1 ? eps : ee[0]; ee[1] = k == 2 ? eps : ee[1]; ee[2] = k == 3 ? eps : ee[2];
      hh[0] = hh[0] || k == 1; hh[1] = hh[1] || k == 2; hh[2] = hh[2] || k == 3;
    }
    ta = tb;
    ya = yb;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    root[k] = rr[k];
    rad[k] = ee[k];
    has[k] = hh[k];
  }
  return ok;
}
// v[i] for an index known only at run time, from values kept in registers
DI float emu_pick6(const float v[6], int i) {
  float r = v[0];
#pragma unroll
  for (int k = 1; k < 6; k++) r = i == k ? v[k] : r;
  return r;
}
// compare-exchange of (key, payload) pairs
DI void emu_cx(float &a, float &ra, float &b, float &rb) {
  if (a > b) {
    float t = a; a = b; b = t;
    t = ra; ra = rb; rb = t;
  }
}
// Root structure of Q on [l,u] (Q(l), Q(u) of certain opposite signs): 1
// with the piece [ra,rb] that holds the one simple root and mu = min |Q'|
// on it; 0 when another root may exist or |Q| may drop to the stopping
// tolerance away from the root piece.  Q' bounds come from its Bernstein
// coefficients on each piece (qb: on [0,1]); dQ, dQp bound the fp32 error of
// Q and Q'.
DI int emu_unique_root(const float n[6], const float qb[5], float l, float u, float ql, float qu, float dQ, float dQp,
                       float stop, float *ra, float *rb, float *mu_out) {
  float sa[8], sb[8], sqa[8], sqb[8];
  int sd[8];
  int sp = 1;
  sa[0] = l; sb[0] = u; sqa[0] = ql; sqb[0] = qu; sd[0] = 0;
  int nroot = 0;
  while (sp > 0) {
    sp--;
    float a = sa[sp], b = sb[sp], qa = sqa[sp], qbv = sqb[sp];
    int d = sd[sp];
    float c[5];
    emu_blossom4(qb, a, b, c);
    float mn = c[0], mx = c[0], amax = fabsf(c[0]);
#pragma unroll
    for (int k = 1; k < 5; k++) { mn = fminf(mn, c[k]); mx = fmaxf(mx, c[k]); amax = fmaxf(amax, fabsf(c[k])); }
    if (mn > dQp || mx < -dQp) {  // Q monotone on the piece
      float mu = (mn > dQp) ? mn - dQp : -mx - dQp;
      if ((qa < 0) != (qbv < 0)) {
        if (++nroot > 1) return 0;
        *ra = a; *rb = b; *mu_out = mu;
      } else if (fminf(fabsf(qa), fabsf(qbv)) <= stop + dQ) {
        return 0;
      }
      continue;
    }
    float m = 0.5f * (a + b);
    float qm = emu_q(n, m);
    float lip = amax + dQp;
    if (fabsf(qm) - lip * 0.5f * (b - a) > stop + dQ) continue;  // no root, |Q| above the stopping tolerance
    if (d >= 6 || sp + 2 > 8) return 0;
    if (fabsf(qm) <= dQ) return 0;
    sa[sp] = m; sb[sp] = b; sqa[sp] = qm; sqb[sp] = qbv; sd[sp] = d + 1; sp++;
    sa[sp] = a; sb[sp] = m; sqa[sp] = qa; sqb[sp] = qm; sd[sp] = d + 1; sp++;
  }
  return nroot == 1;
}
// Called with uniform = true by all 32 lanes of a warp together (lanes
// without a test pass valid = false): the bracket loop then runs a
// warp-wide trip count so the lanes' brackets are decided in step.
// Root structure of the cubic's distance quintic as the reference's walk
// sees it (within_distance.h:150-240): coefficients, breakpoints with
// enclosures, bracket ends and their certain signs.  false when any of it is
// uncertain.
struct EmuRoots {
  float A, n[6], dQ, dQp, qbz[5];
  float ends[6], val[6], qloc[6], bre[6];
  int ne;
  unsigned sc;  // bit j: the bracket of slots j, j + 1 changes sign
};
DI bool emu_root_structure(v2 p0, v2 p1, v2 p2, v2 p3, v2 pt, EmuRoots &R) {
  bool ok = true;
  // distance quintic coefficients exactly as the reference forms them in fp32 (within_distance.h:150-167)
  v2 a = add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3);
  v2 b = add2(sub2(scl2(3, p0), scl2(6, p1)), scl2(3, p2));
  v2 c = add2(scl2(-3, p0), scl2(3, p1));
  v2 e = sub2(p0, pt);
  float A = 3 * sum2(mul2(a, a)), B = 5 * sum2(mul2(a, b)), C = 4 * sum2(mul2(a, c)) + 2 * sum2(mul2(b, b));
  float D = 3 * (sum2(mul2(b, c)) + sum2(mul2(a, e))), E = sum2(mul2(c, c)) + 2 * sum2(mul2(e, b));
  float F = sum2(mul2(e, c));
  float sabs = fabsf(A) + fabsf(B) + fabsf(C) + fabsf(D) + fabsf(E) + fabsf(F);
  if (!(A > 1e-5f * sabs)) ok = false;
  float ia = 1.f / A;
  float n[6] = {1.f, B * ia, C * ia, D * ia, E * ia, F * ia};
  float ns = 1.f + fabsf(n[1]) + fabsf(n[2]) + fabsf(n[3]) + fabsf(n[4]) + fabsf(n[5]);
  float dQ = 1.5e-6f * ns;  // |Q (fp32 here) - Q (fp64 there)| on [0,1]
  float qbz[5];             // Bernstein coefficients of Q' on [0,1]
  {
    float a0 = n[4], a1 = 2 * n[3], a2 = 3 * n[2], a3 = 4 * n[1], a4 = 5.f;
    qbz[0] = a0;
    qbz[1] = a0 + a1 * 0.25f;
    qbz[2] = a0 + a1 * 0.5f + a2 * (1.f / 6.f);
    qbz[3] = a0 + 3 * a1 * 0.25f + a2 * 0.5f + a3 * 0.25f;
    qbz[4] = a0 + a1 + a2 + a3 + a4;
  }
  float dQp = 2e-6f * (5 + 4 * fabsf(n[1]) + 3 * fabsf(n[2]) + 2 * fabsf(n[3]) + fabsf(n[4]));
  // isolator cubic and the bound of its evaluation error
  float mA = 0.4f * fabsf(n[2]) + 0.16f * n[1] * n[1], mB = 0.6f * fabsf(n[3]) + 0.12f * fabsf(n[1] * n[2]);
  float mC = 0.8f * fabsf(n[4]) + 0.08f * fabsf(n[1] * n[3]), mD = fabsf(n[5]) + fabsf(n[1] * n[4]) * 0.04f;
  float pA = 0.4f * n[2] - 0.16f * n[1] * n[1], pB = 0.6f * n[3] - 0.12f * n[1] * n[2];
  float pC = 0.8f * n[4] - 0.08f * n[1] * n[3], pD = n[5] - n[1] * n[4] * 0.04f;
  float del = 1e-6f * (mA + mB + mC + mD) + 1e-30f;
  if (fabsf(pA) <= 1e-6f + 2e-6f * mA) {  // the reference's solver may take its quadratic branch
    del += fabsf(pA) + 2e-6f * mA + 1e-6f;
    pA = 0.f;
  }
  // breakpoints: -B/5 and the isolator's roots, each with its enclosure radius (absent: +inf)
  float qr = -n[1] * 0.2f, eq = 3e-7f * fabsf(qr) + 1e-7f;
  if (fabsf(qr) <= eq || fabsf(qr - 1.f) <= eq) ok = false;
  float bp[5], br[5];
  bool hq = qr > 0.f && qr < 1.f;
  bp[0] = hq ? qr : INFINITY;
  br[0] = hq ? eq : 0.f;
  int nb = hq ? 1 : 0;
  {
    float rts[3], rrad[3];
    bool has[3];
    if (!emu_cubic_roots3(pA, pB, pC, pD, del, rts, rrad, has)) ok = false;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      float rad = rrad[k] + 1.2e-7f;
      if (has[k] && (rts[k] - rad <= 0.f || rts[k] + rad >= 1.f)) ok = false;
      bp[k + 1] = has[k] ? rts[k] : INFINITY;
      br[k + 1] = has[k] ? rad : 0.f;
      nb += has[k] ? 1 : 0;
    }
  }
  bp[4] = 1.f;  // the end t = 1 sorts after every breakpoint, before the absent ones
  br[4] = 0.f;
  // sorting network on the five entries
  emu_cx(bp[0], br[0], bp[1], br[1]); emu_cx(bp[3], br[3], bp[4], br[4]); emu_cx(bp[2], br[2], bp[4], br[4]);
  emu_cx(bp[2], br[2], bp[3], br[3]); emu_cx(bp[0], br[0], bp[3], br[3]); emu_cx(bp[0], br[0], bp[2], br[2]);
  emu_cx(bp[1], br[1], bp[4], br[4]); emu_cx(bp[1], br[1], bp[3], br[3]); emu_cx(bp[1], br[1], bp[2], br[2]);
#pragma unroll
  for (int j = 1; j < 4; j++)
    if (j < nb && bp[j] - bp[j - 1] <= br[j] + br[j - 1]) ok = false;
  // bracket ends (slot 0: t = 0; slots 1..nb: breakpoints; slot nb + 1: t = 1), Q there, and |Q'| within
  // the enclosure of each breakpoint
  int ne = nb + 2;
  float ends[6], val[6], qloc[6], bre[6];
  float qpp = 20 + 12 * fabsf(n[1]) + 6 * fabsf(n[2]) + 2 * fabsf(n[3]);  // |Q''| on [0,1]
#pragma unroll
  for (int j = 0; j < 6; j++) {
    float t = j == 0 ? 0.f : bp[j - 1];
    float rj = j == 0 ? 0.f : br[j - 1];
    float qd = (((5 * t + 4 * n[1]) * t + 3 * n[2]) * t + 2 * n[3]) * t + n[4];
    ends[j] = t;
    bre[j] = rj;
    val[j] = j == 0 ? n[5] : emu_q(n, t);
    qloc[j] = rj > 0.f ? fabsf(qd) + dQp + qpp * rj : 0.f;
    // the sign the reference reads is not certain
    if (j < ne && fabsf(val[j]) <= dQ + qloc[j] * rj) ok = false;
  }
  // brackets whose ends change sign (bit j: slots j, j + 1)
  unsigned sc = 0u;
#pragma unroll
  for (int j = 0; j < 5; j++)
    if (j + 1 < ne && (val[j] < 0) != (val[j + 1] < 0)) sc |= 1u << j;
  R.A = A;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    R.n[k] = n[k];
    R.ends[k] = ends[k];
    R.val[k] = val[k];
    R.qloc[k] = qloc[k];
    R.bre[k] = bre[k];
  }
#pragma unroll
  for (int k = 0; k < 5; k++) R.qbz[k] = qbz[k];
  R.dQ = dQ;
  R.dQp = dQp;
  R.ne = ne;
  R.sc = sc;
  return ok;
}

// The root of Q in the sign-change bracket ending at slot j + 1 of R, as the
// reference's safeguarded Newton iteration finds it (within_distance.h:
// 237-261): ts and a bound eps_t on the distance from ts to where the
// reference stops.  false when the bracket may hold more than one root or
// the iteration may stop next to an end.
DI bool emu_bracket_root(const EmuRoots &R, int j, float &ts, float &eps_t) {
  const float *n = R.n, *qbz = R.qbz;
  float dQ = R.dQ, dQp = R.dQp;
  // lower bracket end: the end of the previous sign-change bracket (the reference keeps its lower end
  // through brackets without a sign change, within_distance.h:237-240)
  unsigned below = R.sc & ((1u << j) - 1u);
  int i0 = below ? 32 - __clz(below) : 0;
  float el = emu_pick6(R.ends, i0), eu = emu_pick6(R.ends, j + 1);
  float vl = emu_pick6(R.val, i0), vu = emu_pick6(R.val, j + 1);
  float rl = emu_pick6(R.bre, i0), ru = emu_pick6(R.bre, j + 1);
  float ql0 = emu_pick6(R.qloc, i0), qu0 = emu_pick6(R.qloc, j + 1);
  // the reference's bracket ends sit within the enclosures of ours: the certain part of the bracket
  float l = el + rl, u = eu - ru;
  // the iteration may stop right at an end where |Q| < 1e-5
  if (fabsf(vl) <= 1e-5f + dQ + 2.f * ql0 * rl || fabsf(vu) <= 1e-5f + dQ + 2.f * qu0 * ru) return false;
  float ql = emu_q(n, l), qu = emu_q(n, u);
  if (fabsf(ql) <= dQ || fabsf(qu) <= dQ || ((ql < 0) == (qu < 0))) return false;
  float ra, rb, mu;
  if (!emu_unique_root(n, qbz, l, u, ql, qu, dQ, dQp, 1e-5f, &ra, &rb, &mu)) return false;
  bool up = emu_q(n, rb) > emu_q(n, ra);
  float lo = ra, hi = rb;
  ts = 0.5f * (ra + rb);
  #pragma unroll 1
  for (int k = 0; k < DVG_EMU_NEWTON; k++) {  // Newton kept inside the root piece
    float y = emu_q(n, ts), dy = (((5 * ts + 4 * n[1]) * ts + 3 * n[2]) * ts + 2 * n[3]) * ts + n[4];
    if ((y > 0) == up) hi = ts; else lo = ts;
    float nt = ts - __fdividef(y, dy);
    ts = (nt >= lo && nt <= hi) ? nt : 0.5f * (lo + hi);
  }
  // how far the root can be from ts: a certified sign change around ts, else the piece
  float er = hi - lo;
  {
    float dts = (((5 * ts + 4 * n[1]) * ts + 3 * n[2]) * ts + 2 * n[3]) * ts + n[4];
    float e2 = fmaxf(2e-7f, __fdividef(2.f * (fabsf(emu_q(n, ts)) + dQ), fmaxf(fabsf(dts), mu)));
    float qm = emu_q(n, ts - e2), qp = emu_q(n, ts + e2);
    if (fabsf(qm) > dQ && fabsf(qp) > dQ && ((qm < 0) != (qp < 0))) er = fminf(er, e2);
  }
  // where the reference may stop: |Q| < 1e-5 around the root, or the 20-step bisection window
  eps_t = __fdividef(1e-5f + dQ, mu) * 1.000001f + er + (eu - el) * 4e-6f + 1e-6f;
  return true;
}

static __device__ __noinline__ int cubic_stroke_decide(bool valid, bool uniform, v2 p0, v2 p1, v2 p2, v2 p3, v2 pt,
                                                       float r0, float r1, float r2, float r3) {
  EmuRoots R;
  int res = emu_root_structure(p0, p1, p2, p3, pt, R) && valid ? -1 : 2;  // -1: not decided yet
  unsigned sc = R.sc;
  float bmax = 3 * sqrtf(fmaxf(fmaxf(distsq2(p0, p1), distsq2(p1, p2)), distsq2(p2, p3)));  // |cubic'|
  float rmaxd = 3 * fmaxf(fmaxf(fabsf(r1 - r0), fabsf(r2 - r1)), fabsf(r3 - r2));  // |radius'|
  float M = fmaxf(fmaxf(absmax2(p0), absmax2(p1)), fmaxf(fmaxf(absmax2(p2), absmax2(p3)), absmax2(pt)));
  bool unsure = false;
  int cnt = res < 0 ? __popc(sc) : 0;
  int rounds = uniform ? __reduce_max_sync(0xffffffffu, cnt) : cnt;
  unsigned rem = sc;
  #pragma unroll 1
  for (int it = 0; it < rounds; it++) {
    if (res >= 0 || it >= cnt) continue;
    int j = __ffs(rem) - 1;
    rem &= rem - 1u;
    float ts, eps_t;
    if (!emu_bracket_root(R, j, ts, eps_t)) {
      unsure = true;
      continue;
    }
    float margin = (bmax + rmaxd) * eps_t + far_margin(M);
    float tt = 1 - ts;
    float rr = (tt * tt * tt) * r0 + (3 * tt * tt * ts) * r1 + (3 * tt * ts * ts) * r2 + (ts * ts * ts) * r3;
    float dd = dist2(eval_cubic(p0, p1, p2, p3, ts), pt);
    if (dd < rr - margin) res = 1;  // the reference returns 1 here or at an earlier bracket
    else if (dd <= rr + margin) unsure = true;
  }
  if (res < 0) res = unsure ? 2 : 0;
  return res;
}

// A cubic segment's control points and the stroke radius at each (per-point
// thickness, or the shape's stroke width), as within_distance.h:143-149 reads them.
struct CubicSeg {
  v2 p[4];
  float r[4];
};
DI CubicSeg cubic_seg(const DevScene &S, int po, int np, int th, int i0, float r) {
  int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
  CubicSeg c;
  c.p[0] = path_pt(S, po, i0);
  c.p[1] = path_pt(S, po, i1);
  c.p[2] = path_pt(S, po, i2);
  c.p[3] = path_pt(S, po, i3);
  c.r[0] = c.r[1] = c.r[2] = c.r[3] = r;
  if (th >= 0) {
    c.r[0] = pget(S, th + i0);
    c.r[1] = pget(S, th + i1);
    c.r[2] = pget(S, th + i2);
    c.r[3] = pget(S, th + i3);
  }
  return c;
}
// The stroke test at a root t of the distance quintic (within_distance.h:262-270).
DI bool cubic_root_hits(const CubicSeg &c, v2 pt, float t) {
  float tt = 1 - t;
  float rr = (tt * tt * tt) * c.r[0] + (3 * tt * tt * t) * c.r[1] + (3 * tt * t * t) * c.r[2] + (t * t * t) * c.r[3];
  return distsq2(eval_cubic(c.p[0], c.p[1], c.p[2], c.p[3], t), pt) < rr * rr;
}
// The brackets of a cubic segment's root walk (within_distance.h:181-261):
// the isolator intervals in order, each one's ends evaluated, the lower end
// kept through intervals without a sign change, the ends of a sign-change
// bracket ordered so that Q rises from lb to ub; the walk stops after the
// bracket that reaches t = 1.  The reference runs quintic_root in each
// bracket in turn and returns at the first root within the stroke, so the
// segment hits exactly when one of these brackets' roots is within it.
// Returns the bracket count (at most 5).
DI int quintic_brackets(const Quintic &q, float lo[5], float hi[5]) {
  float iv[4];
  int ni = quintic_intervals(q, iv);
  float lower = 0.f;
  float ct = NAN;
  double cv = 0.0;
  int nb = 0;
  #pragma unroll 1
  for (int j = 0; j < ni + 1; j++) {
    if (j < ni && iv[j] < 0.f) continue;
    float upper = j < ni ? rmin(iv[j], 1.f) : 1.f;
    float lb = lower, ub = upper;
    double lbe = quintic_eval_cached(q, lb, ct, cv), ube = quintic_eval_cached(q, ub, ct, cv);
    if (lbe * ube > 0) continue;
    if (lbe > ube) { float tmp = lb; lb = ub; ub = tmp; }
    lo[nb] = lb;
    hi[nb] = ub;
    nb++;
    if (upper >= 1.f) break;
    lower = upper;
  }
  return nb;
}

// Root-solve part of the stroke test of one quadratic (nc = 1) or cubic
// (nc = 2) segment, for a point whose end-point checks failed: the
// quadratic's cubic and the cubic's distance quintic, solved as the
// reference does (within_distance.h:95-118, 150-272).  Out of line: it is
// the one fp64-heavy routine, shared by every caller.
static __device__ __noinline__ int segment_root_test(const DevScene &S, int po, int np, int th, int nc, int i0, v2 pt,
                                              float r) {
  if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2);
    float r0 = r, r1 = r, r2 = r;
    if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); r2 = pget(S, th + i2); }
    v2 v = add2(sub2(p0, scl2(2, p1)), p2), w = add2(neg2(p0), p1);
    float A = sum2(mul2(v, v));
    float B = sum2(mul2(scl2(3, v), w));
    float C = sum2(add2(mul2(scl2(2, w), w), mul2(v, sub2(p0, pt))));
    float D = sum2(mul2(w, sub2(p0, pt)));
    float t[3];
    int n = solve_cubic_f(A, B, C, D, t);
    for (int j = 0; j < n; j++) {
      if (t[j] >= 0 && t[j] <= 1) {
        float tt = 1 - t[j];
        float rr = (tt * tt) * r0 + (2 * tt * t[j]) * r1 + (t[j] * t[j]) * r2;
        if (distsq2(eval_quad(p0, p1, p2, t[j]), pt) < rr * rr) return 1;
      }
    }
    return 0;
  }
  CubicSeg c = cubic_seg(S, po, np, th, i0, r);
  Quintic q = cubic_quintic(c.p[0], c.p[1], c.p[2], c.p[3], pt);
  float iv[4];
  int ni = quintic_intervals(q, iv);
  float lower = 0.f;
  float ct = NAN;
  double cv = 0.0;
  #pragma unroll 1
  for (int j = 0; j < ni + 1; j++) {
    if (j < ni && iv[j] < 0.f) continue;
    float upper = j < ni ? rmin(iv[j], 1.f) : 1.f;
    float lb = lower, ub = upper;
    double lbe = quintic_eval_cached(q, lb, ct, cv), ube = quintic_eval_cached(q, ub, ct, cv);
    if (lbe * ube > 0) continue;
    if (lbe > ube) { float tmp = lb; lb = ub; ub = tmp; }
    if (cubic_root_hits(c, pt, quintic_root(q, lb, ub))) return 1;
    if (upper >= 1.f) break;
    lower = upper;
  }
  return 0;
}

// Cheap part of the stroke test of one segment (within_distance.h:20-272):
// lines exactly, quadratic / cubic end points exactly, then the fp32
// outside proof.  1: within, 0: not, -1: the path reports "not within"
// (distance-approximated quadratics), 2: undecided (segment_solve decides).
DN int within_segment_pre(const DevScene &S, int po, int np, int th, int flags, int nc, int i0, int segi, v2 pt,
                          float r) {
  if (nc == 0) {
    int i1 = (i0 + 1) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1);
    float t = dot2(sub2(pt, p0), sub2(p1, p0)) / dot2(sub2(p1, p0), sub2(p1, p0));
    float r0 = r, r1 = r;
    if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); }
    if (t < 0) return distsq2(p0, pt) < r0 * r0 ? 1 : 0;
    if (t > 1) return distsq2(p1, pt) < r1 * r1 ? 1 : 0;
    float rr = r0 + t * (r1 - r0);
    return distsq2(add2(p0, scl2(t, sub2(p1, p0))), pt) < rr * rr ? 1 : 0;
  } else if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2);
    if (flags & 2) {
      v2 cp = quad_closest_approx(p0, p1, p2, pt, nullptr);
      return distsq2(cp, pt) < r * r ? 1 : -1;
    }
    float r0 = r, r1 = r, r2 = r;
    if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); r2 = pget(S, th + i2); }
    if (distsq2(eval_quad(p0, p1, p2, 0), pt) < r0 * r0) return 1;
    if (distsq2(eval_quad(p0, p1, p2, 1), pt) < r2 * r2) return 1;
    float m = fmaxf(fmaxf(absmax2(p0), absmax2(p1)), fmaxf(absmax2(p2), absmax2(pt)));
    const float2 *tp = S.seg_tpts ? S.seg_tpts + (size_t)segi * DVG_TREE_PTS : nullptr;
    const float *tw = S.seg_th ? S.seg_th + (size_t)segi * DVG_TREE_NODES : nullptr;
    return curve_stroke_fast<1>(p0, p1, p2, p2, tp, tw, pt, fmaxf(r0, fmaxf(r1, r2)), far_margin(m)) == 0 ? 0 : 2;
  }
  int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
  v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2), p3 = path_pt(S, po, i3);
  float r0 = r, r1 = r, r2 = r, r3 = r;
  if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); r2 = pget(S, th + i2); r3 = pget(S, th + i3); }
  if (distsq2(eval_cubic(p0, p1, p2, p3, 0), pt) < r0 * r0) return 1;
  if (distsq2(eval_cubic(p0, p1, p2, p3, 1), pt) < r3 * r3) return 1;
  float m = fmaxf(fmaxf(absmax2(p0), absmax2(p1)), fmaxf(fmaxf(absmax2(p2), absmax2(p3)), absmax2(pt)));
  const float2 *tp = S.seg_tpts ? S.seg_tpts + (size_t)segi * DVG_TREE_PTS : nullptr;
  const float *tw = S.seg_th ? S.seg_th + (size_t)segi * DVG_TREE_NODES : nullptr;
  return curve_stroke_fast<2>(p0, p1, p2, p3, tp, tw, pt, fmaxf(fmaxf(r0, r1), fmaxf(r2, r3)), far_margin(m)) == 0 ? 0
                                                                                                               : 2;
}

// fp32 decision of an undecided segment (cubics: cubic_stroke_decide); 2
// when it stays undecided
// uniform: all 32 lanes of the warp call together (valid = false for lanes without a test)
DI int segment_decide(const DevScene &S, int po, int np, int th, int nc, int i0, v2 pt, float r, bool valid = true,
                      bool uniform = false) {
  bool cubic = valid && nc == 2;
  if (!uniform && !cubic) return 2;
  v2 p0 = V2(0.f, 0.f), p1 = p0, p2 = p0, p3 = p0;
  float r0 = r, r1 = r, r2 = r, r3 = r;
  if (cubic) {
    int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
    p0 = path_pt(S, po, i0); p1 = path_pt(S, po, i1); p2 = path_pt(S, po, i2); p3 = path_pt(S, po, i3);
    if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); r2 = pget(S, th + i2); r3 = pget(S, th + i3); }
  }
  int f = cubic_stroke_decide(cubic, uniform, p0, p1, p2, p3, pt, r0, r1, r2, r3);
  return cubic ? f : 2;
}

// an undecided segment, decided: fp32 where that suffices, else the fp64 solve
DI int segment_solve(const DevScene &S, int po, int np, int th, int nc, int i0, v2 pt, float r) {
  int f = segment_decide(S, po, np, th, nc, i0, pt, r);
  return f != 2 ? f : segment_root_test(S, po, np, th, nc, i0, pt, r);
}

// 1: within, 0: not, -1: the path reports "not within" (approx quadratics)
DI int within_segment(const DevScene &S, int s, int po, int np, int th, int flags, int nc, int i0, int segi, v2 pt,
                      float r) {
  int f = within_segment_pre(S, po, np, th, flags, nc, i0, segi, pt, r);
  if (f == 2) f = segment_solve(S, po, np, th, nc, i0, pt, r);
  return f;
}

DN bool within_shape(const DevScene &S, int s, v2 pt, float r) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    float dc = dist2(V2(pget(S, po + 1), pget(S, po + 2)), pt);
    return fabsf(dc - pget(S, po)) < r;
  } else if (kind == DVG_ELLIPSE) {
    flag_error(S, DVG_EFLAG_UNSUPPORTED);  // within_distance.h:343-345 asserts
    return false;
  } else if (kind == DVG_RECT) {
    v2 lt = V2(pget(S, po), pget(S, po + 1)), rt = V2(pget(S, po + 2), pget(S, po + 1));
    v2 lb = V2(pget(S, po), pget(S, po + 3)), rb = V2(pget(S, po + 2), pget(S, po + 3));
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v2 a = k == 0 ? lt : (k == 1 ? lt : (k == 2 ? rt : lb));
      v2 b = k == 0 ? lb : (k == 1 ? rt : rb);
      float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
      if (t < 0) { if (distsq2(a, pt) < r * r) return true; }
      else if (t > 1) { if (distsq2(b, pt) < r * r) return true; }
      else { if (distsq2(add2(a, scl2(t, sub2(b, a))), pt) < r * r) return true; }
    }
    return false;
  }
  int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
  int np = SI(S, s, DVG_SHAPE_NUM_POINTS), th = SI(S, s, DVG_SHAPE_THICKNESS_OFF), flags = SI(S, s, DVG_SHAPE_FLAGS);
  #pragma unroll 1
  for (int k = 0; k < nseg; k++) {
    int seg = S.seg_order[so + k];
    if (nseg > 1 && !box_in_r(S.seg_box[so + seg], pt, S.seg_r[so + seg])) continue;
    int h = within_segment(S, s, po, np, th, flags, __ldg(&S.segment_ctrl[so + seg]), __ldg(&S.seg_point[so + seg]),
                           so + seg, pt, r);
    if (h == 1) return true;
    if (h == -1) return false;
  }
  return false;
}

// within_distance(scene, group, pt, edge_query) (within_distance.h:355-446)
DI bool group_stroke(const DevScene &S, int g, v2 pt, EdgeQ *eq) {
  v2 lp = xform_pt(S.c2s + 9 * g, pt);
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  bool ret = false;
  #pragma unroll 1
  for (int k = 0; k < nsh; k++) {
    int s = __ldg(&S.group_shapes[off + k]);
    float r = stroke_width(S, s);
    if (nsh > 1 && !box_in_r(S.s_box[s], lp, r)) continue;
    if (within_shape(S, s, lp, r)) {
      if (!eq || eq->group != g) return true;
      ret = true;
      if (s == eq->shape) eq->hit = 1;
    }
  }
  return ret;
}

// ---------------------------------------------------------------------------
// closest point / distance (compute_distance.h:12-439)
struct PathInfo { int base_point_id, point_id; float t_root; };

// Closest point of path s to pt within max_radius (closest_point(Path),
// compute_distance.h:26-311), over its segments in visiting order; with
// BANDED, over the band lists that cover pt.y +- max_radius (grown by a
// rounding margin: every segment box_in_r can pass), merged in visiting
// order, so that ties resolve as in the full scan.
template <bool BANDED>
DN bool closest_path_t(const DevScene &S, int s, v2 pt, float max_radius, PathInfo *info, v2 *result) {
  int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF), flags = SI(S, s, DVG_SHAPE_FLAGS);
  float min_dist = max_radius;
  v2 ret = V2(0, 0);
  bool found = false;
  int bi0 = 0, be0 = 0, bi1 = 0, be1 = 0;
  if (BANDED) {
    float slack = max_radius + 1e-5f * (fabsf(pt.y) + max_radius + 1.f);
    if (!band_lists(S, s, pt.y - slack, pt.y + slack, bi0, be0, bi1, be1))
      return closest_path_t<false>(S, s, pt, max_radius, info, result);
  }
  #pragma unroll 1
  for (int k = 0; BANDED || k < nseg; k++) {
    int rank = k;
    if (BANDED && (rank = band_next(S, bi0, be0, bi1, be1)) < 0) break;
    int seg = S.seg_order[so + rank];
    if (nseg > 1 && !box_in_r(S.seg_box[so + seg], pt, min_dist)) continue;
    int nc = __ldg(&S.segment_ctrl[so + seg]), i0 = __ldg(&S.seg_point[so + seg]);
    float dist = 0.f, t_root = 0.f;
    v2 cp = V2(0, 0);
    if (nc == 0) {
      v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, (i0 + 1) % np);
      float t = dot2(sub2(pt, p0), sub2(p1, p0)) / dot2(sub2(p1, p0), sub2(p1, p0));
      if (t < 0) { dist = dist2(p0, pt); cp = p0; t_root = 0; }
      else if (t > 1) { dist = dist2(p1, pt); cp = p1; t_root = 1; }
      else {
        dist = dist2(add2(p0, scl2(t, sub2(p1, p0))), pt);
        cp = add2(p0, scl2(t, sub2(p1, p0)));
        t_root = t;
      }
    } else if (nc == 1) {
      v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1), p2 = path_pt(S, po, (i0 + 2) % np);
      if (flags & 2) {
        cp = quad_closest_approx(p0, p1, p2, pt, &t_root);
        dist = dist2(cp, pt);
      } else {
        float m = fmaxf(fmaxf(absmax2(p0), absmax2(p1)), fmaxf(absmax2(p2), absmax2(pt)));
        const float2 *tp = S.seg_tpts ? S.seg_tpts + (size_t)(so + seg) * DVG_TREE_PTS : nullptr;
        const float *tw = S.seg_th ? S.seg_th + (size_t)(so + seg) * DVG_TREE_NODES : nullptr;
        if (curve_stroke_fast<1>(p0, p1, p2, p2, tp, tw, pt, min_dist, far_margin(m)) == 0) continue;  // cannot improve the best
        v2 pt0 = eval_quad(p0, p1, p2, 0), pt1 = eval_quad(p0, p1, p2, 1);
        float d0 = dist2(pt0, pt), d1 = dist2(pt1, pt);
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
            if (dp < dist) { dist = dp; cp = p; t_root = t[j]; }
          }
        }
      }
    } else {
      v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1), p2 = path_pt(S, po, i0 + 2),
         p3 = path_pt(S, po, (i0 + 3) % np);
      {
        float m = fmaxf(fmaxf(absmax2(p0), absmax2(p1)), fmaxf(fmaxf(absmax2(p2), absmax2(p3)), absmax2(pt)));
        const float2 *tp = S.seg_tpts ? S.seg_tpts + (size_t)(so + seg) * DVG_TREE_PTS : nullptr;
        const float *tw = S.seg_th ? S.seg_th + (size_t)(so + seg) * DVG_TREE_NODES : nullptr;
        if (curve_stroke_fast<2>(p0, p1, p2, p3, tp, tw, pt, min_dist, far_margin(m)) == 0) continue;  // cannot improve the best
      }
      v2 pt0 = eval_cubic(p0, p1, p2, p3, 0), pt1 = eval_cubic(p0, p1, p2, p3, 1);
      float d0 = dist2(pt0, pt), d1 = dist2(pt1, pt);
      dist = d0; cp = pt0; t_root = 0;
      if (d1 < dist) { dist = d1; cp = pt1; t_root = 1; }
      Quintic q = cubic_quintic(p0, p1, p2, p3, pt);
      float iv[4];
      int ni = quintic_intervals(q, iv);
      float lower = 0.f;
      float ct = NAN;
      double cv = 0.0;
      #pragma unroll 1
      for (int j = 0; j < ni + 1; j++) {
        if (j < ni && iv[j] < 0.f) continue;
        float upper = j < ni ? rmin(iv[j], 1.f) : 1.f;
        float lb = lower, ub = upper;
        double lbe = quintic_eval_cached(q, lb, ct, cv), ube = quintic_eval_cached(q, ub, ct, cv);
        if (lbe * ube > 0) continue;
        if (lbe > ube) { float tmp = lb; lb = ub; ub = tmp; }
        float t = quintic_root(q, lb, ub);
        v2 p = eval_cubic(p0, p1, p2, p3, t);
        float dp = dist2(p, pt);
        if (dp < dist) { dist = dp; cp = p; t_root = t; }
        if (upper >= 1.f) break;
        lower = upper;
      }
    }
    if (dist < min_dist) {
      min_dist = dist;
      ret = cp;
      info->base_point_id = seg;
      info->point_id = i0;
      info->t_root = t_root;
      found = true;
    }
  }
  *result = ret;
  return found;
}

// closest_point(shape) (compute_distance.h:313-371)
template <bool BANDED>
DI bool closest_shape_body(const DevScene &S, int s, v2 pt, float max_radius, PathInfo *info, v2 *result) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    // compute_distance.h:18-24 computes the point but reports "not found"
    v2 c = V2(pget(S, po + 1), pget(S, po + 2));
    *result = add2(c, scl2(pget(S, po), normalize2(sub2(pt, c))));
    return false;
  } else if (kind == DVG_ELLIPSE) {
    flag_error(S, DVG_EFLAG_UNSUPPORTED);  // compute_distance.h:362-365 asserts
    return false;
  } else if (kind == DVG_RECT) {
    v2 lt = V2(pget(S, po), pget(S, po + 1)), rt = V2(pget(S, po + 2), pget(S, po + 1));
    v2 lb = V2(pget(S, po), pget(S, po + 3)), rb = V2(pget(S, po + 2), pget(S, po + 3));
    float min_dist = 0.f;
    v2 cp = V2(0, 0);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v2 a = k == 0 ? lt : (k == 1 ? lt : (k == 2 ? rt : lb));
      v2 b = k == 0 ? lb : (k == 1 ? rt : rb);
      bool first = (k == 0);
      float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
      if (t < 0) { float dd = dist2(a, pt); if (first || dd < min_dist) { min_dist = dd; cp = a; } }
      else if (t > 1) { float dd = dist2(b, pt); if (first || dd < min_dist) { min_dist = dd; cp = b; } }
      else {
        // compute_distance.h:333-338 stores p0, not the projection
        float dd = dist2(add2(a, scl2(t, sub2(b, a))), pt);
        if (first || dd < min_dist) { min_dist = dd; cp = a; }
      }
    }
    *result = cp;
    return true;
  }
  if (BANDED && max_radius < INFINITY && __ldg(&S.band_n[s]) > 0)
    return closest_path_t<true>(S, s, pt, max_radius, info, result);
  return closest_path_t<false>(S, s, pt, max_radius, info, result);
}
// scenes with band lists take the BANDED instance (one test at entry, so the
// common instance is unchanged)
DN bool closest_shape_banded(const DevScene &S, int s, v2 pt, float max_radius, PathInfo *info, v2 *result) {
  return closest_shape_body<true>(S, s, pt, max_radius, info, result);
}
DN bool closest_shape(const DevScene &S, int s, v2 pt, float max_radius, PathInfo *info, v2 *result) {
  if (S.band_n) return closest_shape_banded(S, s, pt, max_radius, info, result);
  return closest_shape_body<false>(S, s, pt, max_radius, info, result);
}

// compute_distance (compute_distance.h:373-439)
DI bool group_distance(const DevScene &S, int g, v2 pt, float max_radius, int *min_shape, v2 *closest,
                       PathInfo *info, float *result) {
  v2 lp = xform_pt(S.c2s + 9 * g, pt);
  const float *s2c = S.P + GI(S, g, DVG_GROUP_XFORM_OFF);
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  float min_dist = max_radius;
  bool found = false;
  #pragma unroll 1
  for (int k = 0; k < nsh; k++) {
    int s = __ldg(&S.group_shapes[off + k]);
    if (nsh > 1 && !box_in_r(S.s_box[s], lp, max_radius)) continue;
    PathInfo li;
    li.base_point_id = -1; li.point_id = -1; li.t_root = 0;
    v2 lcp = V2(0, 0);
    if (closest_shape(S, s, lp, max_radius, &li, &lcp)) {
      v2 cp = xform_pt(s2c, lcp);
      float dist = dist2(cp, pt);
      if (!found || dist < min_dist) {
        found = true;
        min_dist = dist;
        if (min_shape) *min_shape = s;
        if (closest) *closest = cp;
        if (info) *info = li;
      }
    }
  }
  *result = min_dist;
  return found;
}

// ---------------------------------------------------------------------------
// paint (diffvg.cpp:276-368)
DI float4 stop_color(const DevScene &S, int co, int i) {
  return F4(pget(S, co + 4 * i), pget(S, co + 4 * i + 1), pget(S, co + 4 * i + 2), pget(S, co + 4 * i + 3));
}
DN float4 paint_color(const DevScene &S, int kind, int off, int nstops, v2 pt) {
  if (kind == DVG_CONSTANT) return F4(pget(S, off), pget(S, off + 1), pget(S, off + 2), pget(S, off + 3));
  float t;
  if (kind == DVG_LINEAR) {
    v2 beg = V2(pget(S, off), pget(S, off + 1)), end = V2(pget(S, off + 2), pget(S, off + 3));
    t = dot2(sub2(pt, beg), sub2(end, beg)) / rmax(dot2(sub2(end, beg), sub2(end, beg)), 1e-3f);
  } else {
    v2 cen = V2(pget(S, off), pget(S, off + 1)), rad = V2(pget(S, off + 2), pget(S, off + 3));
    v2 o = sub2(pt, cen);
    v2 no = V2(o.x / rad.x, o.y / rad.y);
    t = len2(no);
  }
  int oo = off + 4, co = off + 4 + nstops;
  if (t < pget(S, oo)) return stop_color(S, co, 0);
  for (int i = 0; i < nstops - 1; i++) {
    float oc = pget(S, oo + i), on = pget(S, oo + i + 1);
    if (t >= oc && t < on) {
      float4 cc = stop_color(S, co, i), cn = stop_color(S, co, i + 1);
      float tt = (t - oc) / (on - oc);
      return add4(scl4(1 - tt, cc), scl4(tt, cn));
    }
  }
  return stop_color(S, co, nstops - 1);
}

DI void gadd(float *dp, int off, float v) { atomicAdd(dp + off, v); }
// Accumulation of N consecutive parameters that many samples of a warp may
// hit at once (a circle's, ellipse's or rectangle's parameters and group
// transform in the boundary pass; paints and group transforms in the
// interior adjoints, whose warps hold neighbouring pixels): the lanes that
// add to the same block at this point sum their values first and one of them
// adds the sums.  Where the lanes' targets mostly differ (path points in the
// boundary pass) the plain atomics are faster.
template <int N>
DI void gadd_shared(float *dp, int off, const float *v) {
  unsigned peers = __match_any_sync(__activemask(), off);
  if (__popc(peers) == 1) {
#pragma unroll
    for (int k = 0; k < N; k++) atomicAdd(dp + off + k, v[k]);
    return;
  }
  float sum[N];
#pragma unroll
  for (int k = 0; k < N; k++) sum[k] = 0.f;
  for (unsigned m = peers; m; m &= m - 1u) {
    int src = __ffs(m) - 1;
#pragma unroll
    for (int k = 0; k < N; k++) sum[k] += __shfl_sync(peers, v[k], src);
  }
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
#pragma unroll
    for (int k = 0; k < N; k++) atomicAdd(dp + off + k, sum[k]);
  }
}
DI void gadd4(float *dp, int off, float4 v) {
  gadd(dp, off + 0, v.x);
  gadd(dp, off + 1, v.y);
  gadd(dp, off + 2, v.z);
  gadd(dp, off + 3, v.w);
}

// 4 consecutive parameters; with agg, the lanes of the warp that reach this
// point with the same target sum first (gadd_shared)
DI void gadd4_agg(float *dp, int off, float4 v, bool agg) {
  if (agg) {
    float a[4] = {v.x, v.y, v.z, v.w};
    gadd_shared<4>(dp, off, a);
  } else {
    gadd4(dp, off, v);
  }
}

// d_sample_color (diffvg.cpp:370-504).  agg: the samples of the calling warp
// are neighbouring pixels (interior passes), which mostly hit the same paints
DN void d_paint_color(const DevScene &S, int kind, int off, int nstops, v2 pt, float4 d_color, float *dp,
                      float *d_translation, bool agg) {
  if (kind == DVG_CONSTANT) {
    gadd4_agg(dp, off, d_color, agg);
    return;
  }
  int oo = off + 4, co = off + 4 + nstops;
  float t;
  v2 beg = V2(0, 0), end = V2(0, 0), cen = V2(0, 0), rad = V2(0, 0), no = V2(0, 0), o2 = V2(0, 0);
  if (kind == DVG_LINEAR) {
    beg = V2(pget(S, off), pget(S, off + 1)); end = V2(pget(S, off + 2), pget(S, off + 3));
    t = dot2(sub2(pt, beg), sub2(end, beg)) / rmax(dot2(sub2(end, beg), sub2(end, beg)), 1e-3f);
  } else {
    cen = V2(pget(S, off), pget(S, off + 1)); rad = V2(pget(S, off + 2), pget(S, off + 3));
    o2 = sub2(pt, cen);
    no = V2(o2.x / rad.x, o2.y / rad.y);
    t = len2(no);
  }
  if (t < pget(S, oo)) {
    gadd4_agg(dp, co, d_color, agg);
    return;
  }
  for (int i = 0; i < nstops - 1; i++) {
    float oc = pget(S, oo + i), on = pget(S, oo + i + 1);
    if (t >= oc && t < on) {
      float4 cc = stop_color(S, co, i), cn = stop_color(S, co, i + 1);
      float tt = (t - oc) / (on - oc);
      float4 dcc = scl4(1 - tt, d_color), dcn = scl4(tt, d_color);
      float4 diff = sub4(cn, cc);
      float d_tt = d_color.x * diff.x + d_color.y * diff.y + d_color.z * diff.z + d_color.w * diff.w;
      float d_on = -d_tt * tt / (on - oc);
      float d_oc = d_tt * ((tt - 1.f) / (on - oc));
      float d_t = d_tt / (on - oc);
      gadd4_agg(dp, co + 4 * i, dcc, agg);
      gadd4_agg(dp, co + 4 * (i + 1), dcn, agg);
      if (agg) {
        float o2v[2] = {d_oc, d_on};
        gadd_shared<2>(dp, oo + i, o2v);
      } else {
        gadd(dp, oo + i, d_oc);
        gadd(dp, oo + i + 1, d_on);
      }
      if (kind == DVG_LINEAR) {
        float l = rmax(dot2(sub2(end, beg), sub2(end, beg)), 1e-3f);
        v2 d_beg = div2s(scl2(d_t, sub2(neg2(sub2(pt, beg)), sub2(end, beg))), l);
        v2 d_end = div2s(scl2(d_t, sub2(pt, beg)), l);
        float d_l = -d_t * t / l;
        if (dot2(sub2(end, beg), sub2(end, beg)) > 1e-3f) {
          d_beg = add2(d_beg, scl2(2 * d_l, sub2(beg, end)));
          d_end = add2(d_end, scl2(2 * d_l, sub2(end, beg)));
        }
        gadd4_agg(dp, off, F4(d_beg.x, d_beg.y, d_end.x, d_end.y), agg);
        if (d_translation) {
          atomicAdd(d_translation + 0, d_beg.x + d_end.x);
          atomicAdd(d_translation + 1, d_beg.y + d_end.y);
        }
        return;
      } else {
        float l = sqrtf(lensq2(no));
        float d_l_sq = 0.5f * d_t / l;
        v2 d_no = scl2(2 * d_l_sq, no);
        v2 d_off = V2(d_no.x / rad.x, d_no.y / rad.y);
        v2 d_rad = V2(-d_no.x * o2.x / (rad.x * rad.x), -d_no.y * o2.y / (rad.y * rad.y));
        v2 d_cen = neg2(d_off);
        gadd4_agg(dp, off, F4(d_cen.x, d_cen.y, d_rad.x, d_rad.y), agg);
        if (d_translation) {
          atomicAdd(d_translation + 0, d_cen.x);
          atomicAdd(d_translation + 1, d_cen.y);
        }
        // diffvg.cpp:491-498: no return, the last stop also receives d_color
      }
    }
  }
  int last = co + 4 * (nstops - 1);
  gadd4_agg(dp, last, d_color, agg);
}

// d_length / d_normalize (vector.h:496-503, 591-601)
DI v2 d_length2(v2 v, float d_l) {
  float l = sqrtf(lensq2(v));
  float d_l_sq = 0.5f * d_l / l;
  return scl2(2 * d_l_sq, v);
}
DI v2 d_normalize2(v2 v, v2 d_n) {
  float l = len2(v);
  v2 n = div2s(v, l);
  v2 dv = div2s(d_n, l);
  float d_l = -dot2(d_n, n) / l;
  return add2(dv, d_length2(v, d_l));
}
