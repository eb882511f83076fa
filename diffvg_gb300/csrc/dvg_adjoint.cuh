// Device-side adjoints of the closest-point queries and the boundary
// sampler of the GB300 render path (compute_distance.h:442-949,
// sample_boundary.h:9-453, cdf.h:5-29, diffvg.cpp:89-274).
#pragma once

#include "dvg_device.cuh"

// The reference's cos / sin calls on float arguments in the boundary sampler
// evaluate in double precision (the argument is widened, the product with
// the radius stays double until it is stored).
DI double dcos(float x) { return cos((double)x); }
DI double dsin(float x) { return sin((double)x); }

// d_closest_point for paths (compute_distance.h:442-897)
DN void d_closest_path(const DevScene &S, int s, v2 pt, v2 d_cp, const PathInfo &info, float *dp, v2 *d_pt) {
  int np = SI(S, s, DVG_SHAPE_NUM_POINTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  int bp = info.base_point_id, i0 = info.point_id;
  int nc = __ldg(&S.segment_ctrl[so + bp]);
  float t = info.t_root;
  if (nc == 0) {
    int i1 = (i0 + 1) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1);
    float tl = dot2(sub2(pt, p0), sub2(p1, p0)) / dot2(sub2(p1, p0), sub2(p1, p0));
    v2 d0 = V2(0, 0), d1 = V2(0, 0);
    if (tl < 0) d0 = add2(d0, d_cp);
    else if (tl > 1) d1 = add2(d1, d_cp);
    else { d0 = add2(d0, scl2(1 - tl, d_cp)); d1 = add2(d1, scl2(tl, d_cp)); }
    gadd(dp, po + 2 * i0, d0.x); gadd(dp, po + 2 * i0 + 1, d0.y);
    gadd(dp, po + 2 * i1, d1.x); gadd(dp, po + 2 * i1 + 1, d1.y);
  } else if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2);
    v2 d0 = V2(0, 0), d2 = V2(0, 0);
    if (t == 0) d0 = add2(d0, d_cp);
    else if (t == 1) d2 = add2(d2, d_cp);
    else {
      // compute_distance.h:525-580: the control-point adjoints go to
      // block-local shadows and are discarded; only d_pt survives.
      v2 v = add2(sub2(p0, scl2(2, p1)), p2), w = add2(neg2(p0), p1);
      float A = sum2(mul2(v, v));
      float B = sum2(mul2(scl2(3, v), w));
      float C = sum2(add2(mul2(scl2(2, w), w), mul2(v, sub2(p0, pt))));
      v2 d_p = d_cp;
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
    gadd(dp, po + 2 * i0, d0.x); gadd(dp, po + 2 * i0 + 1, d0.y);
    gadd(dp, po + 2 * i2, d2.x); gadd(dp, po + 2 * i2 + 1, d2.y);
  } else {
    int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2), p3 = path_pt(S, po, i3);
    v2 d0 = V2(0, 0), d1 = V2(0, 0), d2 = V2(0, 0), d3 = V2(0, 0);
    if (t == 0) d0 = add2(d0, d_cp);
    else if (t == 1) d3 = add2(d3, d_cp);
    else {
      // The quintic's normalised coefficients and the implicit-function
      // terms below divide by A and by Q'(t) in fp64; one reciprocal of each
      // stands in for the reference's separate divisions (the adjoint moves
      // by fp64 rounding only, far inside the gradient tolerance, and the
      // fp64 divisions are what this routine spends its time on).
      v2 a = add2(sub2(add2(neg2(p0), scl2(3, p1)), scl2(3, p2)), p3);
      v2 b = add2(sub2(scl2(3, p0), scl2(6, p1)), scl2(3, p2));
      v2 c = add2(scl2(-3, p0), scl2(3, p1));
      v2 e = sub2(p0, pt);
      double A = (double)(3 * sum2(mul2(a, a)));
      double inv_a = ddiv(1.0, A);
      Quintic q;
      q.A = A;
      q.B = (double)(5 * sum2(mul2(a, b))) * inv_a;
      q.C = (double)(4 * sum2(mul2(a, c)) + 2 * sum2(mul2(b, b))) * inv_a;
      q.D = (double)(3 * (sum2(mul2(b, c)) + sum2(mul2(a, e)))) * inv_a;
      q.E = (double)(sum2(mul2(c, c)) + 2 * sum2(mul2(e, b))) * inv_a;
      q.F = (double)(sum2(mul2(e, c))) * inv_a;
      v2 d_p = d_cp;
      float tt = 1 - t;
      float d_tt = 3 * tt * tt * dot2(d_p, p0) + 6 * tt * t * dot2(d_p, p1) + 3 * t * t * dot2(d_p, p2);
      float d_t = -d_tt + 3 * tt * tt * dot2(d_p, p1) + 6 * tt * t * dot2(d_p, p2) + 3 * t * t * dot2(d_p, p3);
      d0 = add2(d0, scl2(tt * tt * tt, d_p));
      d1 = add2(d1, scl2(3 * tt * tt * t, d_p));
      d2 = add2(d2, scl2(3 * tt * t * t, d_p));
      d3 = add2(d3, scl2(t * t * t, d_p));
      double pd = quintic_deriv(q, t);
      if (fabs(pd) > 1e-10f) {
        double u = -ddiv(d_t, pd);
        double dF = u, dE = u * t, dD = dE * t, dC = dD * t, dB = dC * t;
        double dA = -(dB * q.B + dC * q.C + dD * q.D + dE * q.E + dF * q.F) * inv_a;
        dB *= inv_a; dC *= inv_a; dD *= inv_a; dE *= inv_a; dF *= inv_a;
        // The control-point terms accumulate in fp32 (the reference adds double
        // products to float accumulators; the two differ by fp32 rounding only,
        // far inside the gradient tolerance, and fp64 runs at a small fraction
        // of the fp32 rate here).
        float fA = (float)dA, fB = (float)dB, fC = (float)dC, fD = (float)dD, fE = (float)dE, fF = (float)dF;
#define ACC(dst, sc, vec) do { float s_ = (sc); (dst).x += s_ * (vec).x; (dst).y += s_ * (vec).y; } while (0)
#define ACC2(dst, s0, v0, s1, v1) do { float a_ = (s0), b_ = (s1); \
    (dst).x += a_ * (v0).x + b_ * (v1).x; (dst).y += a_ * (v0).y + b_ * (v1).y; } while (0)
        ACC(d0, fA * 3 * (-1) * 2, a);
        ACC(d1, fA * 3 * 3 * 2, a);
        ACC(d2, fA * 3 * (-3) * 2, a);
        ACC(d3, fA * 3 * 1 * 2, a);
        ACC(d0, fB * 5, add2(scl2(-1, b), scl2(3, a)));
        ACC(d1, fB * 5, add2(scl2(3, b), scl2(-6, a)));
        ACC(d2, fB * 5, add2(scl2(-3, b), scl2(3, a)));
        ACC(d3, fB * 5, b);
        ACC2(d0, fC * 4, add2(scl2(-1, c), scl2(-3, a)), fC * 2, scl2(3 * 2, b));
        ACC2(d1, fC * 4, add2(scl2(3, c), scl2(3, a)), fC * 2, scl2(-6 * 2, b));
        ACC2(d2, fC * 4, scl2(-3, c), fC * 2, scl2(3 * 2, b));
        ACC(d3, fC * 4, c);
        ACC2(d0, fD * 3, add2(scl2(3, c), scl2(-3, b)), fD * 3, add2(scl2(-1, e), scl2(1, a)));
        ACC2(d1, fD * 3, add2(scl2(-6, c), scl2(3, b)), fD * 3, scl2(3, e));
        ACC2(d2, fD * 3, scl2(3, c), fD * 3, scl2(-3, e));
        ACC(*d_pt, fD * 3, scl2(-1, a));
        ACC2(d0, fE, scl2(-3 * 2, c), fE * 2, add2(scl2(1, b), scl2(3, e)));
        ACC2(d1, fE, scl2(3 * 2, c), fE * 2, scl2(-6, e));
        ACC(d2, fE * 2, scl2(3, e));
        ACC(*d_pt, fE * 2, scl2(-1, b));
        ACC2(d0, fF, scl2(1, c), fF, scl2(-3, e));
        ACC(d1, fF, scl2(3, e));
        ACC(*d_pt, fF, scl2(-1, c));
#undef ACC
#undef ACC2
      }
    }
    gadd(dp, po + 2 * i0, d0.x); gadd(dp, po + 2 * i0 + 1, d0.y);
    gadd(dp, po + 2 * i1, d1.x); gadd(dp, po + 2 * i1 + 1, d1.y);
    gadd(dp, po + 2 * i2, d2.x); gadd(dp, po + 2 * i2 + 1, d2.y);
    gadd(dp, po + 2 * i3, d3.x); gadd(dp, po + 2 * i3 + 1, d3.y);
  }
}

// d_closest_point for rects (compute_distance.h:750-897)
DI void d_closest_rect(const DevScene &S, int po, v2 pt, v2 d_cp, float *dp, v2 *d_pt) {
  v2 lt = V2(pget(S, po), pget(S, po + 1)), rt = V2(pget(S, po + 2), pget(S, po + 1));
  v2 lb = V2(pget(S, po), pget(S, po + 3)), rb = V2(pget(S, po + 2), pget(S, po + 3));
  v2 e0[4] = {lt, lt, rt, lb}, e1[4] = {lb, rt, rb, rb};
  float dd[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v2 a = e0[k], b = e1[k];
    float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
    if (t < 0) dd[k] = dist2(a, pt);
    else if (t > 1) dd[k] = dist2(b, pt);
    else dd[k] = dist2(add2(a, scl2(t, sub2(b, a))), pt);
  }
  int mid = 0;
  float md = dd[0];
  if (dd[1] < md) { md = dd[1]; mid = 1; }
  if (dd[2] < md) { md = dd[2]; mid = 2; }
  if (dd[3] < md) { md = dd[3]; mid = 3; }
  v2 dv[4] = {V2(0, 0), V2(0, 0), V2(0, 0), V2(0, 0)};  // lt, rt, lb, rb
  const int ia[4] = {0, 0, 1, 2}, ib[4] = {2, 1, 3, 3};
  v2 a = e0[mid], b = e1[mid];
  v2 da = V2(0, 0), db = V2(0, 0);
  float t = dot2(sub2(pt, a), sub2(b, a)) / dot2(sub2(b, a), sub2(b, a));
  if (t < 0) da = add2(da, d_cp);
  else if (t > 1) db = add2(db, d_cp);
  else {
    v2 d_p = d_cp;
    da = add2(da, scl2(1 - t, d_p));
    db = add2(db, scl2(t, d_p));
    float d_t = sum2(mul2(d_p, sub2(b, a)));
    float d_num = d_t / dot2(sub2(b, a), sub2(b, a));
    float d_den = d_t * (-t) / dot2(sub2(b, a), sub2(b, a));
    *d_pt = add2(*d_pt, scl2(d_num, sub2(b, a)));
    db = add2(db, scl2(d_num, sub2(pt, a)));
    da = add2(da, scl2(d_num, add2(sub2(a, b), sub2(a, pt))));
    db = add2(db, scl2(d_den, scl2(2, sub2(b, a))));
    da = add2(da, scl2(d_den, scl2(2, sub2(a, b))));
  }
  dv[ia[mid]] = add2(dv[ia[mid]], da);
  dv[ib[mid]] = add2(dv[ib[mid]], db);
  v2 dmin = V2(0, 0), dmax = V2(0, 0);
  dmin = add2(dmin, dv[0]);
  dmax.x += dv[1].x; dmin.y += dv[1].y;
  dmin.x += dv[2].x; dmax.y += dv[2].y;
  dmax = add2(dmax, dv[3]);
  gadd(dp, po + 0, dmin.x); gadd(dp, po + 1, dmin.y); gadd(dp, po + 2, dmax.x); gadd(dp, po + 3, dmax.y);
}

DI void d_closest_shape(const DevScene &S, int s, v2 pt, v2 d_cp, const PathInfo &info, float *dp, v2 *d_pt) {
  int kind = SI(S, s, DVG_SHAPE_KIND), po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  if (kind == DVG_CIRCLE) {
    v2 c = V2(pget(S, po + 1), pget(S, po + 2));
    v2 dn = d_normalize2(sub2(pt, c), scl2(pget(S, po), d_cp));
    v2 d_center = mul2(d_cp, V2(1 + dn.x, 1 + dn.y));
    gadd(dp, po + 1, d_center.x); gadd(dp, po + 2, d_center.y);
    gadd(dp, po + 0, dot2(d_cp, normalize2(sub2(pt, c))));
  } else if (kind == DVG_ELLIPSE) {
    flag_error(S, DVG_EFLAG_UNSUPPORTED);
  } else if (kind == DVG_PATH) {
    d_closest_path(S, s, pt, d_cp, info, dp, d_pt);
  } else {
    d_closest_rect(S, po, pt, d_cp, dp, d_pt);
  }
}

// d_compute_distance (compute_distance.h:899-949)
DI void d_group_distance(const DevScene &S, int g, int s, v2 pt, v2 closest, const PathInfo &info, float d_dist,
                         float *dp, float *d_translation) {
  if (distsq2(pt, closest) < 1e-10f) return;
  const float *c2s = S.c2s + 9 * g;
  int xo = GI(S, g, DVG_GROUP_XFORM_OFF);
  float s2c[9];
#pragma unroll
  for (int i = 0; i < 9; i++) s2c[i] = pget(S, xo + i);
  float c2s_r[9];
#pragma unroll
  for (int i = 0; i < 9; i++) c2s_r[i] = c2s[i];
  v2 lp = xform_pt(c2s_r, pt), lcp = xform_pt(c2s_r, closest);
  v2 d_pt = V2(0, 0), d_cp = V2(0, 0);
  {
    v2 dv = d_length2(sub2(pt, closest), d_dist);
    d_cp = sub2(d_cp, dv);
    d_pt = add2(d_pt, dv);
  }
  v2 d_lcp = V2(0, 0);
  float d_s2c[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  d_xform_pt(s2c, lcp, d_cp, d_s2c, &d_lcp);
  v2 d_lp = V2(0, 0);
  d_closest_shape(S, s, lp, d_lcp, info, dp, &d_lp);
  float d_c2s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  d_xform_pt(c2s_r, pt, d_lp, d_c2s, &d_pt);
  // d_shape_to_canvas += -canvas_to_shape^T * d_canvas_to_shape * canvas_to_shape^T
  float t[9], tmp[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) t[3 * i + j] = c2s_r[3 * j + i];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < 3; k++) acc += (-t[3 * i + k]) * d_c2s[3 * k + j];
      tmp[3 * i + j] = acc;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < 3; k++) acc += tmp[3 * i + k] * t[3 * k + j];
      d_s2c[3 * i + j] += acc;
    }
  gadd_shared<9>(dp, xo, d_s2c);  // the group's transform: every lane of a coherent warp adds here
  if (d_translation) {
    atomicAdd(d_translation + 0, -d_pt.x);
    atomicAdd(d_translation + 1, -d_pt.y);
  }
}

// ---------------------------------------------------------------------------
// edge sampling (sample_boundary.h, cdf.h)
struct BData { int base_point_id, point_id; float t; int is_stroke; };

// sample(cdf, n, u) (cdf.h:5-29)
DI int cdf_sample(const float *cdf, int n, float u, float *updated_u) {
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

DI v2 perturb(v2 ret, v2 *normal, float dir, float r) {
  if (dir != 0.f) {
    ret = add2(ret, scl2(dir * r, *normal));
    if (dir < 0) *normal = neg2(*normal);
  }
  return ret;
}

// per-shape boundary samplers (sample_boundary.h:20-384)
DN v2 sample_shape_boundary(const DevScene &S, int s, float t, v2 *normal, float *pdf, BData *bd, float dir) {
  int kind = SI(S, s, DVG_SHAPE_KIND);
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  float sr = stroke_width(S, s);
  const float TWO_PI = 2 * (float)DVG_PI;
  if (kind == DVG_CIRCLE) {
    float r = pget(S, po);
    v2 c = V2(pget(S, po + 1), pget(S, po + 2));
    v2 off = V2((float)(r * dcos(TWO_PI * t)), (float)(r * dsin(TWO_PI * t)));
    *normal = normalize2(off);
    *pdf /= (TWO_PI * r);
    return perturb(add2(c, off), normal, dir, sr);
  } else if (kind == DVG_ELLIPSE) {
    v2 r = V2(pget(S, po), pget(S, po + 1)), c = V2(pget(S, po + 2), pget(S, po + 3));
    v2 off = V2((float)(r.x * dcos(TWO_PI * t)), (float)(r.y * dsin(TWO_PI * t)));
    float dxdt = (float)(-r.x * dsin(TWO_PI * t) * TWO_PI);
    float dydt = (float)(r.y * dcos(TWO_PI * t) * TWO_PI);
    *normal = normalize2(V2(dydt, -dxdt));
    *pdf /= sqrtf(sq(dxdt) + sq(dydt));
    return perturb(add2(c, off), normal, dir, sr);
  } else if (kind == DVG_RECT) {
    v2 pmin = V2(pget(S, po), pget(S, po + 1)), pmax = V2(pget(S, po + 2), pget(S, po + 3));
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
  // path (sample_boundary.h:80-307)
  int np = SI(S, s, DVG_SHAPE_NUM_POINTS), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
  int th = SI(S, s, DVG_SHAPE_THICKNESS_OFF);
  int closed = SI(S, s, DVG_SHAPE_FLAGS) & 1;
  if (nseg <= 0) { *pdf = 0; return V2(0, 0); }  // a path without segments has no boundary
  if (dir != 0.f && !closed) {
    float cap_length;
    if (th >= 0) cap_length = (float)DVG_PI * (pget(S, th) + pget(S, th + np - 1));
    else cap_length = 2 * (float)DVG_PI * sr;
    float cap_prob = cap_length / (cap_length + S.s_length[s]);
    if (t < cap_prob) {
      t = t / cap_prob;
      *pdf *= cap_prob;
      float r0 = sr, r1 = sr;
      if (th >= 0) { r0 = pget(S, th); r1 = pget(S, th + np - 1); }
      if (dir < 0) {
        v2 p0 = path_pt(S, po, 0);
        v2 off = V2((float)(r0 * dcos(TWO_PI * t)), (float)(r0 * dsin(TWO_PI * t)));
        *normal = normalize2(off);
        *pdf /= (TWO_PI * r0);
        bd->base_point_id = 0; bd->point_id = 0; bd->t = 0;
        return add2(p0, off);
      } else {
        v2 p0 = path_pt(S, po, np - 1);
        v2 off = V2((float)(r1 * dcos(TWO_PI * t)), (float)(r1 * dsin(TWO_PI * t)));
        *normal = normalize2(off);
        *pdf /= (TWO_PI * r1);
        bd->base_point_id = nseg - 1;
        bd->point_id = np - 2 - __ldg(&S.segment_ctrl[so + nseg - 1]);
        bd->t = 1;
        // an open path whose last segment wraps to point 0 has no end cap
        // point here; the reference would index before the path
        if (bd->point_id < 0) { *pdf = 0; return V2(0, 0); }
        return add2(p0, off);
      }
    } else {
      t = (t - cap_prob) / (1 - cap_prob);
      *pdf *= (1 - cap_prob);
    }
  }
  int sid = cdf_sample(S.seg_cdf + so, nseg, t, &t);
  int i0 = __ldg(&S.seg_point[so + sid]);
  int nc = __ldg(&S.segment_ctrl[so + sid]);
  bd->base_point_id = sid; bd->point_id = i0; bd->t = t;
  if (t < -1e-3f || t > 1 + 1e-3f) { *pdf = 0; return V2(0, 0); }
  if (nc == 0) {
    int i1 = (i0 + 1) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1);
    v2 tan = sub2(p1, p0);
    float tl = len2(tan);
    if (tl == 0) { *pdf = 0; return V2(0, 0); }
    *normal = div2s(V2(-tan.y, tan.x), tl);
    *pdf *= S.seg_pmf[so + sid] / tl;
    v2 ret = add2(p0, scl2(t, sub2(p1, p0)));
    if (dir != 0.f) {
      float r0 = sr, r1 = sr;
      if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); }
      float r = r0 + t * (r1 - r0);
      ret = perturb(ret, normal, dir, r);
    }
    return ret;
  } else if (nc == 1) {
    int i1 = i0 + 1, i2 = (i0 + 2) % np;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2);
    v2 tan = add2(scl2(2 * (1 - t), sub2(p1, p0)), scl2(2 * t, sub2(p2, p1)));
    float tl = len2(tan);
    if (tl == 0) { *pdf = 0; return V2(0, 0); }
    *normal = div2s(V2(-tan.y, tan.x), tl);
    *pdf *= S.seg_pmf[so + sid] / tl;
    v2 ret = eval_quad(p0, p1, p2, t);
    if (dir != 0.f) {
      float r0 = sr, r1 = sr, r2 = sr;
      if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); r2 = pget(S, th + i2); }
      float tt = 1 - t;
      float r = (tt * tt) * r0 + (2 * tt * t) * r1 + (t * t) * r2;
      ret = perturb(ret, normal, dir, r);
    }
    return ret;
  }
  int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
  v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i1), p2 = path_pt(S, po, i2), p3 = path_pt(S, po, i3);
  v2 tan = add2(add2(scl2(3 * sq(1 - t), sub2(p1, p0)), scl2(6 * (1 - t) * t, sub2(p2, p1))),
                scl2(3 * t * t, sub2(p3, p2)));
  float tl = len2(tan);
  if (tl == 0) { *pdf = 0; return V2(0, 0); }
  *normal = div2s(V2(-tan.y, tan.x), tl);
  *pdf *= S.seg_pmf[so + sid] / tl;
  v2 ret = eval_cubic(p0, p1, p2, p3, t);
  if (dir != 0.f) {
    float r0 = sr, r1 = sr, r2 = sr, r3 = sr;
    if (th >= 0) { r0 = pget(S, th + i0); r1 = pget(S, th + i1); r2 = pget(S, th + i2); r3 = pget(S, th + i3); }
    float tt = 1 - t;
    float r = (tt * tt * tt) * r0 + (3 * tt * tt * t) * r1 + (3 * tt * t * t) * r2 + (t * t * t) * r3;
    ret = perturb(ret, normal, dir, r);
  }
  return ret;
}

// sample_boundary(scene, ...) (sample_boundary.h:386-453)
DI v2 sample_boundary(const DevScene &S, int g, int s, float t, v2 *normal, float *pdf, BData *bd) {
  *pdf = 1;
  bool has_fill = GI(S, g, DVG_GROUP_FILL_KIND) != DVG_PAINT_NONE;
  bool has_stroke = GI(S, g, DVG_GROUP_STROKE_KIND) != DVG_PAINT_NONE;
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

// accumulate_boundary_gradient (diffvg.cpp:89-274)
DN void accumulate_boundary_gradient(const DevScene &S, int g, int s, float contrib, float t, v2 normal,
                                     const BData &bd, v2 local_pt, float *dp) {
  int kind = SI(S, s, DVG_SHAPE_KIND), po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  int th = kind == DVG_PATH ? SI(S, s, DVG_SHAPE_THICKNESS_OFF) : -1;
  int np = kind == DVG_PATH ? SI(S, s, DVG_SHAPE_NUM_POINTS) : 0;
  int so = kind == DVG_PATH ? SI(S, s, DVG_SHAPE_SEG_OFF) : 0;
  if (bd.is_stroke) {
    if (th >= 0) {
      int i0 = bd.point_id;
      float tt = bd.t;
      int nc = __ldg(&S.segment_ctrl[so + bd.base_point_id]);
      if (nc == 0) {
        int i1 = (i0 + 1) % np;
        gadd(dp, th + i0, (1 - tt) * contrib); gadd(dp, th + i1, (tt) * contrib);
      } else if (nc == 1) {
        int i1 = i0 + 1, i2 = (i0 + 2) % np;
        gadd(dp, th + i0, sq(1 - tt) * contrib);
        gadd(dp, th + i1, (2 * (1 - tt) * tt) * contrib);
        gadd(dp, th + i2, (tt * tt) * contrib);
      } else {
        int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
        gadd(dp, th + i0, ((1 - tt) * (1 - tt) * (1 - tt)) * contrib);
        gadd(dp, th + i1, 3 * sq(1 - tt) * tt * contrib);
        gadd(dp, th + i2, 3 * (1 - tt) * tt * tt * contrib);
        gadd(dp, th + i3, tt * tt * tt * contrib);
      }
    } else {
      gadd(dp, SI(S, s, DVG_SHAPE_STROKE_WIDTH_OFF), contrib);
    }
  }
  if (kind == DVG_CIRCLE) {
    const float d[3] = {contrib, normal.x * contrib, normal.y * contrib};
    gadd_shared<3>(dp, po, d);
  } else if (kind == DVG_ELLIPSE) {
    const float d[4] = {(float)(dcos(2 * (float)DVG_PI * t) * normal.x * contrib),
                        (float)(dsin(2 * (float)DVG_PI * t) * normal.y * contrib), normal.x * contrib,
                        normal.y * contrib};
    gadd_shared<4>(dp, po, d);
  } else if (kind == DVG_PATH) {
    int i0 = bd.point_id;
    float tt = bd.t;
    int nc = __ldg(&S.segment_ctrl[so + bd.base_point_id]);
    if (nc == 0) {
      int i1 = (i0 + 1) % np;
      gadd(dp, po + 2 * i0 + 0, (1 - tt) * normal.x * contrib); gadd(dp, po + 2 * i0 + 1, (1 - tt) * normal.y * contrib);
      gadd(dp, po + 2 * i1 + 0, (tt) * normal.x * contrib); gadd(dp, po + 2 * i1 + 1, (tt) * normal.y * contrib);
    } else if (nc == 1) {
      int i1 = i0 + 1, i2 = (i0 + 2) % np;
      gadd(dp, po + 2 * i0 + 0, sq(1 - tt) * normal.x * contrib);
      gadd(dp, po + 2 * i0 + 1, sq(1 - tt) * normal.y * contrib);
      gadd(dp, po + 2 * i1 + 0, (2 * (1 - tt) * tt) * normal.x * contrib);
      gadd(dp, po + 2 * i1 + 1, (2 * (1 - tt) * tt) * normal.y * contrib);
      gadd(dp, po + 2 * i2 + 0, (tt * tt) * normal.x * contrib);
      gadd(dp, po + 2 * i2 + 1, (tt * tt) * normal.y * contrib);
    } else {
      int i1 = i0 + 1, i2 = i0 + 2, i3 = (i0 + 3) % np;
      float c0 = (1 - tt) * (1 - tt) * (1 - tt);
      gadd(dp, po + 2 * i0 + 0, c0 * normal.x * contrib); gadd(dp, po + 2 * i0 + 1, c0 * normal.y * contrib);
      gadd(dp, po + 2 * i1 + 0, 3 * sq(1 - tt) * tt * normal.x * contrib);
      gadd(dp, po + 2 * i1 + 1, 3 * sq(1 - tt) * tt * normal.y * contrib);
      gadd(dp, po + 2 * i2 + 0, 3 * (1 - tt) * tt * tt * normal.x * contrib);
      gadd(dp, po + 2 * i2 + 1, 3 * (1 - tt) * tt * tt * normal.y * contrib);
      gadd(dp, po + 2 * i3 + 0, tt * tt * tt * normal.x * contrib);
      gadd(dp, po + 2 * i3 + 1, tt * tt * tt * normal.y * contrib);
    }
  } else {
    if (normal.x == -1 && normal.y == 0) gadd(dp, po + 0, -contrib);
    else if (normal.x == 1 && normal.y == 0) gadd(dp, po + 2, contrib);
    else if (normal.x == 0 && normal.y == -1) gadd(dp, po + 1, -contrib);
    else if (normal.x == 0 && normal.y == 1) gadd(dp, po + 3, contrib);
    else flag_error(S, DVG_EFLAG_UNSUPPORTED);  // diffvg.cpp:253-256 asserts
  }
  float d_s2c[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  v2 d_local = V2(0, 0);
  int xo = GI(S, g, DVG_GROUP_XFORM_OFF);
  float s2c[9];
#pragma unroll
  for (int i = 0; i < 9; i++) s2c[i] = pget(S, xo + i);
  d_xform_pt(s2c, local_pt, scl2(contrib, normal), d_s2c, &d_local);
  if (kind == DVG_PATH) {  // paths: samples spread over many shapes and groups
#pragma unroll
    for (int i = 0; i < 9; i++) gadd(dp, xo + i, d_s2c[i]);
  } else {  // one circle, ellipse or rectangle takes every sample of its boundary
    gadd_shared<9>(dp, xo, d_s2c);
  }
}
