// Scene preparation kernels of the GB300 render path.
//
// The reference rebuilds its scene on the host on every call
// (scene.cpp:919-998: boxes, per-path segment BVHs, group BVHs, length
// CDFs).  Here the topology stays resident on the device and everything
// that depends on the parameter values is derived by these kernels from the
// parameter arena, so an optimisation step never leaves the GPU:
//   k_group_xform   canvas_to_shape = inverse(shape_to_canvas)   (shape.h:123)
//   k_shape_prep    boxes and boundary lengths of circles, ellipses, rects
//   k_path_prep     path and segment boxes and stroke radii, the per-path
//                   segment visiting order, boundary lengths and per-path
//                   segment CDFs (scene.cpp:113-333, 495-625), a warp a path
//   k_group_prep    group boxes, max stroke radius, tile range (scene.cpp:627-684)
//   k_sampling_cdf  the (group, shape) boundary-length CDF (scene.cpp:207-246)
//   k_bin_count / k_bin_scan / k_bin_fill
//                   per-16x16-tile candidate group lists in ascending group
//                   id, replacing the reference's top-level group BVH.
#include "dvg_internal.h"

namespace dvg {

__global__ void k_group_xform(DevScene S) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= S.num_groups) return;
  float m[9], r[9];
  int xo = GI(S, g, DVG_GROUP_XFORM_OFF);
  for (int i = 0; i < 9; i++) m[i] = S.P[xo + i];
  inverse3(m, r);
  for (int i = 0; i < 9; i++) S.c2s[9 * g + i] = r[i];
}

// Stable bottom-up merge sort of idx[0..n) by key[idx] (ties keep index order).
__device__ void sort_by_key_stable(int *idx, int *tmp, const float *key, int n) {
  for (int width = 1; width < n; width *= 2) {
    for (int lo = 0; lo < n; lo += 2 * width) {
      int mid = min(lo + width, n), hi = min(lo + 2 * width, n);
      int a = lo, b = mid, o = lo;
      while (a < mid && b < hi) {
        if (key[idx[b]] < key[idx[a]]) tmp[o++] = idx[b++];
        else tmp[o++] = idx[a++];
      }
      while (a < mid) tmp[o++] = idx[a++];
      while (b < hi) tmp[o++] = idx[b++];
    }
    for (int i = 0; i < n; i++) idx[i] = tmp[i];
  }
}

// Visiting order of a path's segments: segments sorted by box y-centre and
// paired bottom-up into a binary tree (scene.cpp:439-494, 602-620), leaves
// visited depth-first with child1 before child0 (the stack discipline of
// winding_number.h:44-172).  scratch holds 10*n + 8 ints.
__device__ void path_leaf_order(const float4 *boxes, int n, int *out, int *scratch) {
  int *idx = scratch;
  float *key = reinterpret_cast<float *>(scratch + n);
  int *tmp = scratch + 2 * n;
  int *c0 = scratch + 3 * n;
  int *c1 = scratch + 5 * n;
  int *stack = scratch + 7 * n;
  for (int i = 0; i < n; i++) { idx[i] = i; key[i] = 0.5f * (boxes[i].y + boxes[i].w); }
  sort_by_key_stable(idx, tmp, key, n);
  if (n == 1) { out[0] = idx[0]; return; }
  int size = 2 * n - 1;
  for (int i = 0; i < size; i++) { c0[i] = -1; c1[i] = -1; }
  int prev_beg = 0, prev_end = n;
  int leftover = prev_end % 2 == 0 ? -1 : prev_end - 1;
  while (prev_end - prev_beg >= 1 || leftover != -1) {
    int length = (prev_end - prev_beg) / 2;
    if ((prev_end - prev_beg) % 2 == 1 && leftover != -1 && leftover != prev_end - 1) length += 1;
    for (int i = 0; i < length; i++) {
      int a = prev_beg + 2 * i, b = prev_beg + 2 * i + 1;
      if (b >= prev_end) { b = leftover; leftover = -1; }
      c0[prev_end + i] = a;
      c1[prev_end + i] = b;
    }
    if (length == 1 && leftover == -1) break;
    prev_beg = prev_end;
    prev_end = prev_beg + length;
    if (length % 2 == 1 && leftover == -1) leftover = prev_end - 1;
  }
  int sp = 0, k = 0;
  stack[sp++] = size - 1;
  while (sp > 0 && k < n) {
    int node = stack[--sp];
    if (node < n) { out[k++] = idx[node]; continue; }
    if (sp + 2 > 3 * n) break;  // cannot happen for a tree of 2n-1 nodes
    stack[sp++] = c0[node];
    stack[sp++] = c1[node];
  }
}

// path_leaf_order with the 32 lanes of a warp (all call it; the same
// result).  The stable sort by key runs as bottom-up merge passes in which
// every element finds its place by a binary search in the other run (left
// elements count the right run's smaller keys, right elements the left
// run's smaller or equal keys: the stable merge).  The pairing tree depends
// on n only: its levels are replayed in every lane, each level's nodes are
// filled by the lanes with their parent links and leaf counts, and a leaf's
// place in the depth-first visit (child1 before child0) is the sum of the
// leaf counts of the child1 siblings of the ancestors it reaches through
// child0.  Keys with a NaN make the order depend on the merge sequence
// itself: lane 0 then runs path_leaf_order.  scratch holds 10*n + 8 ints.
__device__ void path_leaf_order_warp(const float4 *boxes, int n, int *out, int *scratch, int lane) {
  const unsigned full = 0xffffffffu;
  int *idx = scratch;
  float *key = reinterpret_cast<float *>(scratch + n);
  int *tmp = scratch + 2 * n;
  bool nan = false;
  for (int i = lane; i < n; i += 32) {
    float k = 0.5f * (boxes[i].y + boxes[i].w);
    key[i] = k;
    idx[i] = i;
    nan |= !(k == k);
  }
  if (__any_sync(full, nan)) {
    __syncwarp();
    if (lane == 0) path_leaf_order(boxes, n, out, scratch);
    __syncwarp();
    return;
  }
  __syncwarp();
  if (n == 1) {
    if (lane == 0) out[0] = 0;
    __syncwarp();
    return;
  }
  int *src = idx, *dst = tmp;
  for (int w = 1; w < n; w *= 2) {
    for (int i = lane; i < n; i += 32) {
      int lo = i / (2 * w) * (2 * w), mid = min(lo + w, n), hi = min(lo + 2 * w, n);
      int v = src[i];
      float kv = key[v];
      int pos;
      if (i < mid) {  // right-run elements with a smaller key come first
        int a = mid, b = hi;
        while (a < b) {
          int m = (a + b) >> 1;
          if (key[src[m]] < kv) a = m + 1; else b = m;
        }
        pos = i + (a - mid);
      } else {  // left-run elements with a smaller or equal key come first
        int a = lo, b = mid;
        while (a < b) {
          int m = (a + b) >> 1;
          if (key[src[m]] <= kv) a = m + 1; else b = m;
        }
        pos = lo + (i - mid) + (a - lo);
      }
      dst[pos] = v;
    }
    __syncwarp();
    int *t = src; src = dst; dst = t;
  }
  // src: the segments in sorted order (sorted position -> segment)
  int size = 2 * n - 1, root = size - 1;
  int *c0 = scratch + 3 * n, *c1 = scratch + 5 * n, *par = scratch + 7 * n;
  // leaf counts of the tree's nodes, over the buffers the sort no longer needs: [n, 3n) when the
  // sorted order is in idx = [0, n), else [0, 2n) (it is then in tmp = [2n, 3n))
  int *cnt = src == idx ? scratch + n : scratch;
  const int *sorted = src;
  for (int i = lane; i < n; i += 32) cnt[i] = 1;
  if (lane == 0) par[root] = -1;
  __syncwarp();
  int prev_beg = 0, prev_end = n;
  int leftover = prev_end % 2 == 0 ? -1 : prev_end - 1;
  for (int guard = 0; guard < 2 * n + 2 && (prev_end - prev_beg >= 1 || leftover != -1); guard++) {
    int length = (prev_end - prev_beg) / 2;
    if ((prev_end - prev_beg) % 2 == 1 && leftover != -1 && leftover != prev_end - 1) length += 1;
    for (int i = lane; i < length; i += 32) {
      int a = prev_beg + 2 * i, b = prev_beg + 2 * i + 1;
      if (b >= prev_end) b = leftover;
      int v = prev_end + i;
      c0[v] = a;
      c1[v] = b;
      par[a] = v;
      par[b] = v;
      cnt[v] = cnt[a] + cnt[b];
    }
    __syncwarp();
    if (length > 0 && prev_beg + 2 * (length - 1) + 1 >= prev_end) leftover = -1;
    if (length == 1 && leftover == -1) break;
    prev_beg = prev_end;
    prev_end = prev_beg + length;
    if (length % 2 == 1 && leftover == -1) leftover = prev_end - 1;
  }
  for (int leaf = lane; leaf < n; leaf += 32) {
    int pos = 0, v = leaf;
    for (int guard = 0; v != root && guard < size; guard++) {
      int u = par[v];
      if (u < 0) break;
      if (c0[u] == v) pos += cnt[c1[u]];
      v = u;
    }
    out[pos] = sorted[leaf];
  }
  __syncwarp();
}

// Boxes, radii, lengths, CDFs of the non-path shapes (one thread per shape);
// paths are k_path_prep's.
__global__ void k_shape_prep(DevScene S) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S.num_shapes) return;
  int kind = SI(S, s, DVG_SHAPE_KIND);
  if (kind == DVG_PATH) return;
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  const float *p = S.P + po;
  float L = 0.f;
  if (kind == DVG_CIRCLE) {
    float r = p[0];
    v2 c = V2(p[1], p[2]);
    S.s_box[s] = F4(c.x - r, c.y - r, c.x + r, c.y + r);
    L += (float)(2.f * DVG_PI) * r;
  } else if (kind == DVG_ELLIPSE) {
    v2 r = V2(p[0], p[1]), c = V2(p[2], p[3]);
    S.s_box[s] = F4(c.x - r.x, c.y - r.y, c.x + r.x, c.y + r.y);
    float a = r.x, b = r.y;
    L += (float)((float)DVG_PI * (3 * (a + b) - sqrt((double)((3 * a + b) * (a + 3 * b)))));
  } else if (kind == DVG_RECT) {
    S.s_box[s] = F4(p[0], p[1], p[2], p[3]);
    L += 2 * (p[2] - p[0] + p[3] - p[1]);
  }
  S.s_length[s] = L;
}

// Path shapes (one warp per path): the shape box, each segment's box and
// stroke radius, the segments' visiting order, the boundary length and the
// per-segment length CDF (scene.cpp:113-333, 495-625).  Lanes work on
// segments; the sums whose rounding depends on their order (the length and
// the CDF) run in segment order in lane 0, so every value is the one a
// sequential pass forms.
__global__ void k_path_prep(DevScene S) {
  const unsigned full = 0xffffffffu;
  int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (s >= S.num_shapes || SI(S, s, DVG_SHAPE_KIND) != DVG_PATH) return;
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF);
  int np = SI(S, s, DVG_SHAPE_NUM_POINTS), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS);
  int so = SI(S, s, DVG_SHAPE_SEG_OFF), th = SI(S, s, DVG_SHAPE_THICKNESS_OFF);
  // shape box: point 0, grown by the others (box_add skips a NaN point once the box is a number, so
  // the NaN-skipping extremes of points 1.. give the sequential result)
  float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  for (int i = 1 + lane; i < np; i += 32) {
    v2 q = path_pt(S, po, i);
    mnx = fminf(mnx, q.x);
    mny = fminf(mny, q.y);
    mxx = fmaxf(mxx, q.x);
    mxy = fmaxf(mxy, q.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(full, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(full, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(full, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(full, mxy, o));
  }
  if (lane == 0) {
    float4 b = box_empty();
    if (np > 0) {
      v2 q = path_pt(S, po, 0);
      b = F4(rmin(mnx, q.x), rmin(mny, q.y), rmax(mxx, q.x), rmax(mxy, q.y));
    }
    S.s_box[s] = b;
  }
  float r = stroke_width(S, s);
  for (int i = lane; i < nseg; i += 32) {
    int nc = S.segment_ctrl[so + i], pid = S.seg_point[so + i];
    float4 sb = box_empty();
    float rr = r;
    for (int k = 0; k <= nc + 1; k++) {
      int id = (k == nc + 1) ? (pid + k) % np : pid + k;
      sb = box_add(sb, path_pt(S, po, id));
      if (th >= 0) {
        float rk = S.P[th + id];
        rr = (k == 0) ? rk : rmax(rr, rk);
      }
    }
    S.seg_box[so + i] = sb;
    S.seg_r[so + i] = rr;
  }
  __syncwarp();
  if (nseg > 0) path_leaf_order_warp(S.seg_box + so, nseg, S.seg_order + so, S.scratch + 10 * so + 8 * s, lane);
  // per-segment lengths (the 3- / 4-point polylines), then their sum in segment order
  for (int i = lane; i < nseg; i += 32) {
    int nc = S.segment_ctrl[so + i], i0 = S.seg_point[so + i];
    float t;
    if (nc == 0) {
      t = dist2(path_pt(S, po, (i0 + 1) % np), path_pt(S, po, i0));
    } else if (nc == 1) {
      v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1), p2 = path_pt(S, po, (i0 + 2) % np);
      v2 v1 = eval_quad(p0, p1, p2, 0.5f);
      t = dist2(v1, p0) + dist2(v1, p2);
    } else {
      v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1), p2 = path_pt(S, po, i0 + 2),
         p3 = path_pt(S, po, (i0 + 3) % np);
      v2 v1 = eval_cubic(p0, p1, p2, p3, 1.f / 3.f), v2_ = eval_cubic(p0, p1, p2, p3, 2.f / 3.f);
      t = dist2(v1, p0) + dist2(v1, v2_) + dist2(v2_, p3);
    }
    S.seg_pmf[so + i] = t;  // the length for now; the pmf below
  }
  __syncwarp();
  float L = 0.f;
  if (lane == 0) {
    float len = 0.f;
    for (int i = 0; i < nseg; i++) len += S.seg_pmf[so + i];
    L += len;
  }
  L = __shfl_sync(full, L, 0);
  float inv = 1.f / L;
  for (int i = lane; i < nseg; i += 32) S.seg_pmf[so + i] = S.seg_pmf[so + i] * inv;
  __syncwarp();
  if (lane == 0) {
    float cdf = 0.f;
    for (int i = 0; i < nseg; i++) {
      float dd = S.seg_pmf[so + i];
      cdf = (i == 0) ? dd : dd + cdf;
      S.seg_cdf[so + i] = cdf;
    }
    S.s_length[s] = L;
  }
}

// y-band segment lists of the long paths (one warp per path): the path's
// box is cut into bands of equal height (as many as fit at least
// DVG_BAND_MIN_HEIGHT, at most shape_band.x), and every segment is
// listed, by its visiting rank in ascending order, in each band from
// band_of(its box's top) to band_of(its bottom).  The reference culls a path's segments with a
// y-sorted segment BVH (scene.cpp:602-620, walked in winding_number.h:54-172
// and compute_distance.h:36-300); the band lists give a point's candidates as
// one contiguous list.  A path whose lists would pass their capacity, or
// whose box has no finite positive height, gets none this call (band_n 0):
// its queries scan every segment, with the same results.  Lanes find each
// rank's band range, count the bands' entries, and then each lane fills its
// own bands in rank order.
__global__ void k_band_fill(DevScene S) {
  const unsigned full = 0xffffffffu;
  int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (s >= S.num_shapes) return;
  int4 sb = S.shape_band[s];
  if (sb.x <= 0) return;
  if (lane == 0) S.band_n[s] = 0;
  float4 box = S.s_box[s];
  float h = box.w - box.y;
  if (!(h > 0.f) || !(h < INFINITY)) return;
  // bands at least DVG_BAND_MIN_HEIGHT tall (shape units), at most sb.x of them
  int nb = (int)fminf((float)sb.x, fmaxf(1.f, floorf(h / DVG_BAND_MIN_HEIGHT)));
  float inv = (float)nb / h;
  if (!(inv < INFINITY)) return;
  float2 geo = make_float2(box.y, inv);
  if (lane == 0) S.band_geo[s] = geo;
  int so = SI(S, s, DVG_SHAPE_SEG_OFF), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS);
  int *st = S.band_start + sb.y;
  int *out = S.band_seg + sb.z;
  int2 *range = reinterpret_cast<int2 *>(S.scratch + 10 * so + 8 * s);  // [nseg] band range of rank k
  for (int b = lane; b <= nb; b += 32) st[b] = 0;
  __syncwarp();
  long long total = 0;
  for (int k = lane; k < nseg; k += 32) {
    float4 q = S.seg_box[so + S.seg_order[so + k]];
    int b0 = 1, b1 = 0;  // a NaN box passes no box test: no band
    if (q.y == q.y && q.w == q.w) {
      b0 = band_of(geo, nb, q.y);
      b1 = band_of(geo, nb, q.w);
      for (int b = b0; b <= b1; b++) atomicAdd(&st[b], 1);
      total += b1 - b0 + 1;
    }
    range[k] = make_int2(b0, b1);
  }
  for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(full, total, o);
  __syncwarp();
  if (total > sb.w) return;
  if (lane == 0) {  // counts -> starts; st[nb] = the entry count
    for (int b = 0, run = 0; b <= nb; b++) {
      int c = b < nb ? st[b] : 0;
      st[b] = run;
      run += c;
    }
  }
  __syncwarp();
  for (int b = lane; b < nb; b += 32) {  // each lane fills its bands, ranks ascending
    int w = st[b];
    for (int k = 0; k < nseg; k++) {
      int2 r = range[k];
      if (r.x <= b && b <= r.y) out[w++] = k;
    }
  }
  __syncwarp();
  if (lane == 0) S.band_n[s] = nb;
}

__device__ __forceinline__ int clamp_tile(double f, int hi, bool lower) {
  // clamps a floored tile coordinate to the grid (first / last tile)
  if (lower) return f < 0 ? 0 : (f > hi - 1 ? hi : (int)f);
  return f > hi - 1 ? hi - 1 : (f < 0 ? -1 : (int)f);
}

// Tabulated subdivision trees of the curved path segments (one warp per
// shape, lanes over its segments): the curve points at t = k / 2^D and the
// hull width of every piece of levels 0..D, formed exactly as the outside
// proof forms them (curve_stroke_fast).
__global__ void k_seg_tree(DevScene S) {
  int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (s >= S.num_shapes || !S.seg_tpts || SI(S, s, DVG_SHAPE_KIND) != DVG_PATH) return;
  int po = SI(S, s, DVG_SHAPE_PARAM_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
  int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
  for (int i = lane; i < nseg; i += 32) {
    int nc = S.segment_ctrl[so + i], i0 = S.seg_point[so + i];
    if (nc != 1 && nc != 2) continue;
    float2 *tp = S.seg_tpts + (size_t)(so + i) * DVG_TREE_PTS;
    float *th = S.seg_th + (size_t)(so + i) * DVG_TREE_NODES;
    v2 p0 = path_pt(S, po, i0), p1 = path_pt(S, po, i0 + 1);
    v2 p2 = path_pt(S, po, nc == 2 ? i0 + 2 : (i0 + 2) % np), p3 = nc == 2 ? path_pt(S, po, (i0 + 3) % np) : p2;
    const float step = __int_as_float((127 - DVG_TREE_DEPTH) << 23);  // 2^-D
    for (int k = 0; k < DVG_TREE_PTS; k++) {
      float t = (float)k * step;
      tp[k] = nc == 2 ? cubic_blossom(p0, p1, p2, p3, t, t, t) : quad_blossom(p0, p1, p2, t, t);
    }
    th[0] = 0.f;
    for (unsigned node = 1; node < DVG_TREE_NODES; node++) {
      int d = 31 - __clz(node);
      float scale = __int_as_float((127 - d) << 23);
      float ta = (float)(node - (1u << d)) * scale, tb = ta + scale;
      th[node] = nc == 2 ? cubic_hull_width(cubic_blossom(p0, p1, p2, p3, ta, ta, ta),
                                            cubic_blossom(p0, p1, p2, p3, ta, ta, tb),
                                            cubic_blossom(p0, p1, p2, p3, ta, tb, tb),
                                            cubic_blossom(p0, p1, p2, p3, tb, tb, tb))
                         : quad_hull_width(quad_blossom(p0, p1, p2, ta, ta), quad_blossom(p0, p1, p2, ta, tb),
                                           quad_blossom(p0, p1, p2, tb, tb));
    }
  }
}

// Stroke records: the stroke tests of every stroke group flattened into one
// array, group after group, each group's shapes in order and each path's
// segments in visiting order (seg_order), one record per segment; a shape
// that is not a path, or a path with distance-approximated segments, gets
// one record for the whole shape.  A record holds the cull box (the
// segment's box grown by its stroke radius, or the shape's when a cull
// applies to the whole shape), the indices a test needs and the first record
// of the next shape, so that the sample loops test segments without
// following indices through the scene tables.
DI int stroke_record_count(const DevScene &S, int g) {
  if (GI(S, g, DVG_GROUP_STROKE_KIND) == DVG_PAINT_NONE) return 0;
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF), n = 0;
  for (int k = 0; k < nsh; k++) {
    int s = S.group_shapes[off + k];
    bool per_segment = SI(S, s, DVG_SHAPE_KIND) == DVG_PATH && !(SI(S, s, DVG_SHAPE_FLAGS) & 2);
    n += per_segment ? SI(S, s, DVG_SHAPE_NUM_SEGMENTS) : 1;
  }
  return n;
}

// exclusive scan of the per-group record counts (one block of 1024 threads)
__global__ void k_rec_scan(DevScene S) {
  int G = S.num_groups;
  __shared__ int part[1024];
  int per = (G + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(lo + per, G);
  int sum = 0;
  for (int g = lo; g < hi; g++) sum += stroke_record_count(S, g);
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x > 0 ? part[threadIdx.x - 1] : 0;
  for (int g = lo; g < hi; g++) {
    int c = stroke_record_count(S, g);
    S.g_rec[g] = make_int2(run, run + c);
    run += c;
  }
}

// canvas box of a shape-space box under the group's shape_to_canvas, one
// pixel wider (the group boxes of k_group_prep are formed the same way)
DI float4 canvas_box_of(const float *m, float4 b) {
  if (!(b.x > -INFINITY && b.y > -INFINITY && b.z < INFINITY && b.w < INFINITY))
    return F4(-INFINITY, -INFINITY, INFINITY, INFINITY);
  float4 cb = box_empty();
  cb = box_add(cb, xform_pt(m, V2(b.x, b.y)));
  cb = box_add(cb, xform_pt(m, V2(b.x, b.w)));
  cb = box_add(cb, xform_pt(m, V2(b.z, b.y)));
  cb = box_add(cb, xform_pt(m, V2(b.z, b.w)));
  return F4(cb.x - 1.f, cb.y - 1.f, cb.z + 1.f, cb.w + 1.f);
}

__global__ void k_rec_fill(DevScene S) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= S.num_groups) return;
  int j = S.g_rec[g].x;
  if (S.g_rec[g].y <= j) return;
  const float4 all = F4(-INFINITY, -INFINITY, INFINITY, INFINITY);
  float m9[9];
  const float *xm = S.P + GI(S, g, DVG_GROUP_XFORM_OFF);
  for (int i = 0; i < 9; i++) m9[i] = xm[i];
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  for (int k = 0; k < nsh; k++) {
    int s = S.group_shapes[off + k];
    float r = stroke_width(S, s);
    int po = SI(S, s, DVG_SHAPE_PARAM_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
    int th = SI(S, s, DVG_SHAPE_THICKNESS_OFF);
    bool per_segment = SI(S, s, DVG_SHAPE_KIND) == DVG_PATH && !(SI(S, s, DVG_SHAPE_FLAGS) & 2);
    float4 sb = S.s_box[s];
    float4 shape_cull = nsh > 1 ? F4(sb.x - r, sb.y - r, sb.z + r, sb.w + r) : all;
    if (!per_segment) {
      S.rec_box[j] = shape_cull;
      S.rec_cbox[j] = canvas_box_of(m9, shape_cull);
      S.rec_a[j] = make_int4(-1, s, 0, 0);
      S.rec_b[j] = make_int4(po, np, th, j + 1);
      S.rec_r[j] = r;
      j++;
      continue;
    }
    int nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, s, DVG_SHAPE_SEG_OFF);
    int next = j + nseg;
    for (int m = 0; m < nseg; m++, j++) {
      int seg = S.seg_order[so + m];
      float4 b = S.seg_box[so + seg];
      float rr = S.seg_r[so + seg];
      S.rec_box[j] = nseg > 1 ? F4(b.x - rr, b.y - rr, b.z + rr, b.w + rr) : shape_cull;
      S.rec_cbox[j] = canvas_box_of(m9, S.rec_box[j]);
      S.rec_a[j] = make_int4(so + seg, s, S.segment_ctrl[so + seg], S.seg_point[so + seg]);
      S.rec_b[j] = make_int4(po, np, th, next);
      S.rec_r[j] = r;
    }
  }
}

__global__ void k_group_prep(DevScene S, int4 *g_tile_range) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= S.num_groups) return;
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  float4 b = box_empty();
  float max_r = 0.f;
  for (int k = 0; k < nsh; k++) {
    int s = S.group_shapes[off + k];
    b = (k == 0) ? S.s_box[s] : box_union(b, S.s_box[s]);
    float r = stroke_width(S, s);
    if (SI(S, s, DVG_SHAPE_KIND) == DVG_PATH && SI(S, s, DVG_SHAPE_THICKNESS_OFF) >= 0 &&
        SI(S, s, DVG_SHAPE_NUM_SEGMENTS) > 0) {
      // the reference reads node 0 of the path BVH: the leaf with the lowest y-centre
      int so = SI(S, s, DVG_SHAPE_SEG_OFF), nseg = SI(S, s, DVG_SHAPE_NUM_SEGMENTS);
      int best = 0;
      float bk = 0.5f * (S.seg_box[so].y + S.seg_box[so].w);
      for (int i = 1; i < nseg; i++) {
        float ki = 0.5f * (S.seg_box[so + i].y + S.seg_box[so + i].w);
        if (ki < bk) { bk = ki; best = i; }
      }
      r = S.seg_r[so + best];
    }
    max_r = (k == 0) ? r : (max_r < r ? r : max_r);
  }
  S.g_local_box[g] = b;
  const float *m = S.P + GI(S, g, DVG_GROUP_XFORM_OFF);
  float mm[9];
  for (int i = 0; i < 9; i++) mm[i] = m[i];
  float4 cb = box_empty();
  cb = box_add(cb, xform_pt(mm, V2(b.x, b.y)));
  cb = box_add(cb, xform_pt(mm, V2(b.x, b.w)));
  cb = box_add(cb, xform_pt(mm, V2(b.z, b.y)));
  cb = box_add(cb, xform_pt(mm, V2(b.z, b.w)));
  S.g_canvas_box[g] = cb;
  float r = GI(S, g, DVG_GROUP_STROKE_KIND) == DVG_PAINT_NONE ? 0.f : max_r;
  S.g_max_radius[g] = r;
  // tiles touched by the box grown by the stroke radius and one pixel
  int4 tr;
  if (S.num_groups == 1) {
    tr = make_int4(0, S.tiles_x - 1, 0, S.tiles_y - 1);
  } else {
    double fx0 = floor(((double)cb.x - r - 1.0) / DVG_TILE), fx1 = floor(((double)cb.z + r + 1.0) / DVG_TILE);
    double fy0 = floor(((double)cb.y - r - 1.0) / DVG_TILE), fy1 = floor(((double)cb.w + r + 1.0) / DVG_TILE);
    if (!(fx0 <= fx1) || !(fy0 <= fy1)) {
      tr = make_int4(1, 0, 1, 0);
    } else {
      tr = make_int4(clamp_tile(fx0, S.tiles_x, true), clamp_tile(fx1, S.tiles_x, false),
                     clamp_tile(fy0, S.tiles_y, true), clamp_tile(fy1, S.tiles_y, false));
    }
  }
  g_tile_range[g] = tr;
}

// Boundary-length CDF over (group, shape) pairs in group order, normalised
// (scene.cpp:207-246).  The running sum keeps the reference's sequential
// summation order: the block stages the lengths in shared memory and one
// thread accumulates them; normalisation is parallel.
__global__ void k_sampling_cdf(DevScene S) {
  __shared__ float buf[1024];
  __shared__ float carry;
  __shared__ int bad;
  int nt = S.num_total;
  if (threadIdx.x == 0) { carry = 0.f; bad = 0; }
  for (int base = 0; base < nt; base += 1024) {
    int m = min(1024, nt - base);
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) buf[j] = S.s_length[S.smp_shape[base + j]];
    __syncthreads();
    if (threadIdx.x == 0) {
      float cdf = carry;
      for (int j = 0; j < m; j++) {
        float len = buf[j];
        cdf = (base + j == 0) ? len : len + cdf;
        buf[j] = cdf;
      }
      carry = cdf;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      S.smp_cdf[base + j] = buf[j];
      S.smp_pmf[base + j] = S.s_length[S.smp_shape[base + j]];
    }
  }
  __syncthreads();
  if (nt <= 0) return;
  float norm = carry;
  if (threadIdx.x == 0) {
    if (norm <= 0) { atomicOr(S.err, DVG_EFLAG_SCENE_ZERO); bad = 1; }
    else if (!isfinite(norm)) { atomicOr(S.err, DVG_EFLAG_SCENE_NAN); bad = 1; }
  }
  __syncthreads();
  if (bad) return;
  for (int i = threadIdx.x; i < nt; i += blockDim.x) { S.smp_cdf[i] /= norm; S.smp_pmf[i] /= norm; }
}

__device__ __forceinline__ bool tile_hit(int4 r, int tx, int ty) {
  return tx >= r.x && tx <= r.y && ty >= r.z && ty <= r.w;
}

// one block per tile: number of candidate groups
// Whether group g enters the candidate list of tile (tx, ty), and the mask
// of its stroke records that may reach the tile (tile_mask).  A group whose
// box reaches the tile enters unless it has no fill and none of its stroke
// records reaches the tile.
DI bool tile_keep(const DevScene &S, const int4 *g_tile_range, int g, int tx, int ty, unsigned *mask) {
  *mask = 0u;
  if (!tile_hit(g_tile_range[g], tx, ty)) return false;
  int2 rg = S.g_rec[g];
  float x0 = (float)(tx * DVG_TILE), y0 = (float)(ty * DVG_TILE);
  float x1 = x0 + (float)DVG_TILE, y1 = y0 + (float)DVG_TILE;
  unsigned m = 0u;
  int csh = rec_chunk_shift(rg.y - rg.x);
  for (int j = rg.x; j < rg.y; j++) {
    int bit = (j - rg.x) >> csh;
    if (m & (1u << bit)) {  // the rest of this chunk cannot add to the mask
      j = rg.x + ((bit + 1) << csh) - 1;
      continue;
    }
    float4 b = S.rec_cbox[j];
    if (b.x <= x1 && b.z >= x0 && b.y <= y1 && b.w >= y0) m |= 1u << bit;
  }
  *mask = m;
  return m != 0u || GI(S, g, DVG_GROUP_FILL_KIND) != DVG_PAINT_NONE;
}

__global__ void k_bin_count(DevScene S, const int4 *g_tile_range, int *tile_count) {
  int t = blockIdx.x;
  int tx = t % S.tiles_x, ty = t / S.tiles_x;
  int c = 0;
  unsigned mask;
  for (int g = threadIdx.x; g < S.num_groups; g += blockDim.x) c += tile_keep(S, g_tile_range, g, tx, ty, &mask) ? 1 : 0;
  __shared__ int red[32];
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int sum = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) sum += red[w];
    tile_count[t] = sum;
  }
}

// exclusive scan of the tile counts (one block of 1024 threads)
__global__ void k_bin_scan(DevScene S, const int *tile_count, int tile_cap, int *bin_total) {
  int T = S.tiles_x * S.tiles_y;
  __shared__ int part[1024];
  int per = (T + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(lo + per, T);
  int sum = 0;
  for (int i = lo; i < hi; i++) sum += tile_count[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int total = part[blockDim.x - 1];
  bool overflow = total > tile_cap;
  int run = threadIdx.x > 0 ? part[threadIdx.x - 1] : 0;
  for (int i = lo; i < hi; i++) {
    S.tile_start[i] = overflow ? 0 : run;
    run += tile_count[i];
  }
  if (threadIdx.x == 0) {
    S.tile_start[T] = overflow ? 0 : total;
    *bin_total = total;
    if (overflow) atomicOr(S.err, DVG_EFLAG_BIN_OVERFLOW);
  }
}

// one block per tile: ordered (ascending group id) compaction of the hits
__global__ void k_bin_fill(DevScene S, const int4 *g_tile_range) {
  if (*(volatile unsigned *)S.err & DVG_EFLAG_BIN_OVERFLOW) return;
  int t = blockIdx.x;
  int tx = t % S.tiles_x, ty = t / S.tiles_x;
  __shared__ int warp_cnt[32];
  __shared__ int base_sh;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) base_sh = S.tile_start[t];
  __syncthreads();
  for (int g0 = 0; g0 < S.num_groups; g0 += blockDim.x) {
    int g = g0 + threadIdx.x;
    unsigned mask = 0u;
    bool hit = g < S.num_groups && tile_keep(S, g_tile_range, g, tx, ty, &mask);
    unsigned m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) warp_cnt[wid] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < nw; w++) {
      int c = warp_cnt[w];
      if (w < wid) before += c;
      total += c;
    }
    if (hit) {
      int at = base_sh + before + __popc(m & ((1u << lane) - 1u));
      S.tile_list[at] = g;
      S.tile_mask[at] = mask;
    }
    __syncthreads();
    if (threadIdx.x == 0) base_sh += total;
    __syncthreads();
  }
}

cudaError_t launch_prepare(const DevScene &S, int tile_cap, int *bin_total, int4 *g_tile_range, int *tile_count,
                           cudaStream_t st) {
  int G = S.num_groups, NS = S.num_shapes;
  int T = S.tiles_x * S.tiles_y;
  if (G > 0) k_group_xform<<<(G + 127) / 128, 128, 0, st>>>(S);
  if (NS > 0) k_shape_prep<<<(NS + 63) / 64, 64, 0, st>>>(S);
  if (NS > 0 && S.num_paths > 0) k_path_prep<<<(NS + 3) / 4, 128, 0, st>>>(S);
  if (NS > 0 && S.num_segments > 0 && S.seg_tpts) k_seg_tree<<<(NS + 3) / 4, 128, 0, st>>>(S);
  if (NS > 0 && S.shape_band) k_band_fill<<<(NS + 3) / 4, 128, 0, st>>>(S);
  if (G > 0) k_group_prep<<<(G + 127) / 128, 128, 0, st>>>(S, g_tile_range);
  if (G > 0 && S.num_records > 0) {  // without stroke records g_rec keeps the zeros it was created with
    k_rec_scan<<<1, 1024, 0, st>>>(S);
    k_rec_fill<<<(G + 127) / 128, 128, 0, st>>>(S);
  }
  k_sampling_cdf<<<1, 256, 0, st>>>(S);
  k_bin_count<<<T, 128, 0, st>>>(S, g_tile_range, tile_count);
  k_bin_scan<<<1, 1024, 0, st>>>(S, tile_count, tile_cap, bin_total);
  k_bin_fill<<<T, 128, 0, st>>>(S, g_tile_range);
  return cudaGetLastError();
}

}  // namespace dvg
