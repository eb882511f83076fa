// Per-sample colour evaluation of the GB300 render path: the forward blend,
// its reverse-mode adjoint, the prefiltered (analytic coverage) variant and
// the signed distance query (diffvg.cpp:525-833, 835-1113, 709-775).
//
// Candidate groups come from the sample's 16x16 canvas tile list in
// ascending group id, which is the reference's back-to-front fragment order
// (it sorts fragments by group id, diffvg.cpp:605-615), so the forward pass
// blends each fragment as soon as it is found and keeps no fragment list.
// The adjoint gathers the fragments of its sample into a per-thread list and
// walks it in reverse; it takes them from the forward pass's per-sample
// cache when that is valid for the current parameters and re-evaluates them
// otherwise.
#pragma once

#include "dvg_adjoint.cuh"

#include <cstddef>
#include <type_traits>

// Sample position of sample idx (diffvg.cpp:1164-1180).
DI v2 sample_pos(const DevRender &R, int idx, bool prefilter, int &x, int &y) {
  Pcg rng = pcg_init(idx, R.seed);
  int sx = idx % R.nsx;
  int sy = (idx / R.nsx) % R.nsy;
  x = (idx / (R.nsx * R.nsy)) % R.w;
  y = (idx / (R.nsx * R.nsy * R.w));
  float rx = pcg_float(rng), ry = pcg_float(rng);
  if (prefilter) { rx = 0.5f; ry = 0.5f; }
  return V2(x + ((float)sx + rx) / R.nsx, y + ((float)sy + ry) / R.nsy);
}

// gather_d_color (diffvg.cpp:777-815)
DI float4 gather_d_color(const DevRender &R, v2 pt) {
  int x = (int)pt.x, y = (int)pt.y;
  float4 d = F4(0, 0, 0, 0);
  for (int dy = -R.ri; dy <= R.ri; dy++)
    for (int dx = -R.ri; dx <= R.ri; dx++) {
      int xx = x + dx, yy = y + dy;
      if (xx >= 0 && xx < R.w && yy >= 0 && yy < R.h) {
        float xc = xx + 0.5f, yc = yy + 0.5f;
        float fw = filter_weight(R.ftype, R.fr, xc - pt.x, yc - pt.y);
        float ws = R.weight[yy * R.w + xx];
        if (ws > 0) {
          float4 di = __ldg(reinterpret_cast<const float4 *>(R.d_image) + (yy * R.w + xx));
          d = add4(d, scl4(fw / ws, di));
        }
      }
    }
  return d;
}

DI void blend(float4 &acc, float4 c) {
  float na = c.w;
  acc.x = acc.x * (1 - na) + na * c.x;
  acc.y = acc.y * (1 - na) + na * c.y;
  acc.z = acc.z * (1 - na) + na * c.z;
  acc.w = acc.w * (1 - na) + na;
}

DI float4 finish_color(float4 acc) {
  if (acc.w > 1e-6f) { acc.x /= acc.w; acc.y /= acc.w; acc.z /= acc.w; }
  return acc;
}

// ---------------------------------------------------------------------------
// Warp-batched root solves.  Each lane first runs the cheap part of every
// stroke test of its sample (exact end-point and line checks, fp32 outside
// proofs); segments that stay undecided become jobs in the warp's queue in
// shared memory.  The warp then solves all queued jobs together, one job per
// lane, so the fp64 root solves run with full warps instead of the few lanes
// whose sample happens to sit near a curve.  Each lane finally blends its
// fragments in group order with the solved results.  Every lane of the warp
// must call the batched functions (inactive lanes pass active = false).
#ifndef DVG_LANE_JOBS
#define DVG_LANE_JOBS 8
#endif
// jobs per lane of the wide queues: the forward and boundary walks of
// stroke-heavy scenes, whose samples queue more segment tests than 8 often
// enough that the overflow (decided one lane at a time) costs more than the
// shared memory the larger queue takes from L1
#ifndef DVG_LANE_JOBS_WIDE
#define DVG_LANE_JOBS_WIDE 12
#endif
// Candidate fragments a lane holds before the warp decides and blends them
// (its column of the warp's fragment front, in shared memory).  A group adds
// at most two (its stroke and its fill).
#ifndef DVG_FRONT
#define DVG_FRONT 16
#endif
struct SegJob { int shape, seg; float x, y, r; };

// candidate fragment of a sample: key = 2 * group + is_stroke; meta bit 31
// = decided hit, else bits 0-7 / 8-15 = the lane's job range whose results
// decide it
struct FragRef { int key, meta; };
#define DVG_META_HIT (1 << 31)

template <int CAP>
struct WarpQueueT {
  static constexpr int kJobs = CAP;
  // a job's number in the warp's queue
  typedef typename std::conditional<(32 * CAP <= 256), unsigned char, unsigned short>::type JobNum;
  SegJob job[32][CAP];
  unsigned result[32];
  int offs[33];
  JobNum pend[32 * CAP];                   // jobs the fp32 decision left open
  unsigned pend_lanes;                     // lanes that own one of them
  int qid[32];                             // the lanes' query numbers (deferral)
  // lane l's candidate fragments in front[0..nf)[l] (SharedFront).  Last, so
  // that kernels whose lanes keep their fronts themselves (LocalFront) give
  // each warp only the part before it (queue_local_bytes).
  FragRef front[DVG_FRONT][32];
};
typedef WarpQueueT<DVG_LANE_JOBS> WarpQueue;
typedef WarpQueueT<DVG_LANE_JOBS_WIDE> WarpQueueWide;
static_assert(DVG_LANE_JOBS <= 31 && DVG_LANE_JOBS_WIDE <= 31,
              "a lane's jobs are bits of a 32-bit mask and of an 8-bit range");
// bytes of a warp queue without its shared fragment front, rounded to 16
template <class Q>
__host__ __device__ constexpr int queue_local_bytes() {
  return (int)((offsetof(Q, front) + 15) / 16 * 16);
}

// A lane's fragment front: its column of the warp queue's front in shared
// memory (the interior adjoint, which keeps at most 16 hits itself), or
// an array of DVG_LOCAL_FRONT entries of its own (the forward and boundary
// passes: deep samples then rarely make the warp decide its jobs early).
struct SharedFront {
  static constexpr int kCap = DVG_FRONT;
  WarpQueue *q;
  int lane;
  DI SharedFront(WarpQueue *q_, int lane_) : q(q_), lane(lane_) {}
  DI FragRef &operator[](int i) const { return q->front[i][lane]; }
};
#ifndef DVG_LOCAL_FRONT
#define DVG_LOCAL_FRONT 64
#endif
struct LocalFront {
  static constexpr int kCap = DVG_LOCAL_FRONT;
  FragRef f[DVG_LOCAL_FRONT];
  DI LocalFront(const void *, int) {}
  DI FragRef &operator[](int i) { return f[i]; }
  DI const FragRef &operator[](int i) const { return f[i]; }
};

// owner lane and slot of the warp's j-th queued job
template <class Q>
DI const SegJob &warp_job(const Q *q, int j, int &owner, int &idx) {
  int lo = 0, hi = 31;  // last lane with offs <= j
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (q->offs[mid] <= j) lo = mid; else hi = mid - 1;
  }
  owner = lo;
  idx = j - q->offs[lo];
  return q->job[lo][idx];
}

// Decide every queued job of the warp, spread over its lanes, with the fp32
// decision; the jobs it leaves open are listed in q->pend (their owners in
// q->pend_lanes).  Returns how many (the same in every lane).
template <class Q>
DI int warp_decide(const DevScene &S, Q *q, int lane, int njobs) {
  const unsigned full = 0xffffffffu;
  int incl = njobs;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  int total = __shfl_sync(full, incl, 31);
  q->offs[lane] = incl - njobs;
  if (lane == 31) q->offs[32] = total;
  q->result[lane] = 0u;
  if (lane == 0) q->pend_lanes = 0u;
  __syncwarp();
  int npend = 0;
  #pragma unroll 1
  for (int base = 0; base < total; base += 32) {  // warp-uniform trip count
    int j = base + lane;
    bool valid = j < total;
    int owner = 0, idx = 0;
    SegJob jb = valid ? warp_job(q, j, owner, idx) : SegJob{0, 0, 0.f, 0.f, 0.f};
    int s = jb.shape;
    int f = segment_decide(S, valid ? SI(S, s, DVG_SHAPE_PARAM_OFF) : 0, valid ? SI(S, s, DVG_SHAPE_NUM_POINTS) : 1,
                           valid ? SI(S, s, DVG_SHAPE_THICKNESS_OFF) : -1,
                           valid ? __ldg(&S.segment_ctrl[jb.seg]) : 0, valid ? __ldg(&S.seg_point[jb.seg]) : 0,
                           V2(jb.x, jb.y), jb.r, valid, true);  // all lanes: the decisions run in step
    if (valid && f == 1) atomicOr(&q->result[owner], 1u << idx);
    bool pending = valid && f == 2;
    unsigned bal = __ballot_sync(full, pending);
    if (pending) {
      q->pend[npend + __popc(bal & ((1u << lane) - 1u))] = (typename Q::JobNum)j;
      atomicOr(&q->pend_lanes, 1u << owner);
    }
    npend += __popc(bal);
  }
  __syncwarp();
  return npend;
}

// The fp64 solves of the warp's open jobs, compacted so that as many lanes
// as there are jobs run them together.
template <class Q>
DI void warp_fp64(const DevScene &S, Q *q, int lane, int npend) {
  #pragma unroll 1
  for (int k = lane; k < npend; k += 32) {
    int owner, idx;
    SegJob jb = warp_job(q, q->pend[k], owner, idx);
    int s = jb.shape;
    int hit = segment_root_test(S, SI(S, s, DVG_SHAPE_PARAM_OFF), SI(S, s, DVG_SHAPE_NUM_POINTS),
                                SI(S, s, DVG_SHAPE_THICKNESS_OFF), __ldg(&S.segment_ctrl[jb.seg]),
                                __ldg(&S.seg_point[jb.seg]), V2(jb.x, jb.y), jb.r);
    if (hit) atomicOr(&q->result[owner], 1u << idx);
  }
  __syncwarp();
}

// Decide every queued job of the warp: the fp32 decision first, then the
// fp64 solve of the jobs it left open.
template <class Q>
DI void warp_solve(const DevScene &S, Q *q, int lane, int njobs) {
  warp_fp64(S, q, lane, warp_decide(S, q, lane, njobs));
}

DI bool frag_hit(int meta, unsigned res) {
  if (meta & DVG_META_HIT) return true;
  int lo = meta & 255, hi = (meta >> 8) & 255;
  unsigned mask = (hi - lo >= 32) ? 0xffffffffu : ((1u << (hi - lo)) - 1u);
  return ((res >> lo) & mask) != 0u;
}

// Pass 1 of a sample: candidate fragments in group order, undecided stroke
// segments queued.
//
// All 32 lanes of the warp call it (lanes without a sample pass active =
// false) and walk the candidates together: the groups of the lanes' tile
// lists in ascending order (a merge of the lists: the lanes of a warp mostly
// share one tile), and inside a stroke group its records (its shapes'
// segments with their cull boxes, in the order of the nested loops of
// within_distance, within_distance.h:355-446, and sample_color,
// diffvg.cpp:525-585).  Each lane tests its own point; the records' loads and
// the loop control are shared, and the segment tests of the lanes whose
// culls pass run together.  A shape that hits ends the lane's walk of that
// shape (and of its group, outside the group of an edge query) as the
// reference's early returns do.
//
// The lane's candidate fragments go to its column of the warp's fragment
// front.  Before a group that could overfill a lane's front, every lane
// hands the decided fragments at the start of its front to
// flush(count, 0, 0) and keeps the rest; if a lane's front is still too
// full, the warp decides its queued jobs, every active lane hands its whole
// front to flush(nf, results, eq_jobs) and starts an empty one, and flushed
// is set (the same in every lane).  Returns the
// number of fragments left in the lane's front; overflow is set when the
// sample has more than DVG_MAX_FRAGMENTS candidates (diffvg.cpp:542).
template <class Q, class Front, class Flush>
DI int collect_fragments(const DevScene &S, v2 pt, Q *q, Front &front, int lane, int &njobs, EdgeQ *eq,
                         unsigned &eq_jobs, bool &overflow, bool &flushed, bool active, Flush &flush) {
  const unsigned full = 0xffffffffu;
  int k = 0, e = 0;
  bool list = true;
  if (active) list = cand_range(S, pt, k, e);
  const int G = S.num_groups;
  int nf = 0, total = 0;
  auto emit = [&](int key, int meta) {
    if (total < DVG_MAX_FRAGMENTS) {
      front[nf++] = FragRef{key, meta};
      total++;
    } else {
      overflow = true;
    }
  };
  auto fill = [&](int gg) {
    if (GI(S, gg, DVG_GROUP_FILL_KIND) != DVG_PAINT_NONE && group_inside(S, gg, pt, eq)) emit(2 * gg, DVG_META_HIT);
  };
  #pragma unroll 1
  while (true) {
    int myg = k < e ? (list ? __ldg(&S.tile_list[k]) : k) : 0x7fffffff;
    int g = __reduce_min_sync(full, myg);
    if (g == 0x7fffffff) break;
    if (__any_sync(full, nf > Front::kCap - 2)) {
      // first hand over each lane's decided prefix (fills decide during the
      // walk); only a front still full after that waits for the warp's jobs
      int u = 0;
      while (u < nf && (front[u].meta & DVG_META_HIT)) u++;
      if (active && u > 0) flush(u, 0u, 0u);
      for (int i = u; i < nf; i++) front[i - u] = front[i];
      nf -= u;
      if (__any_sync(full, nf > Front::kCap - 2)) {
        warp_solve(S, q, lane, njobs);
        if (active) flush(nf, q->result[lane], eq_jobs);
        nf = 0;
        njobs = 0;
        eq_jobs = 0u;
        flushed = true;
      }
    }
    bool act = myg == g;
    unsigned tmask = act ? (list ? __ldg(&S.tile_mask[k]) : full) : 0u;
    if (act) k++;
    if (act && G > 1 && !box_in_r(S.g_canvas_box[g], pt, S.g_max_radius[g])) act = false;
    if (!__any_sync(full, act)) continue;
    int2 rg = __ldg(&S.g_rec[g]);
    unsigned um = __reduce_or_sync(full, act ? tmask : 0u);
    if (rg.y <= rg.x || um == 0u) {  // no stroke record of the group reaches these tiles
      if (act) fill(g);
      continue;
    }
    // stroke records of g, walked together
    v2 lp = act ? xform_pt(S.c2s + 9 * g, pt) : pt;
    int glo = njobs, cs = -1, slo = njobs, skip_to = rg.x;
    bool live = act, gret = false, mark = false;
    bool is_eq = act && eq && eq->group == g;
    int jb = rg.x, j = rg.x, csh = rec_chunk_shift(rg.y - rg.x);
    #pragma unroll 1
    while (j < rg.y) {
      // skip the chunks of records that cannot reach the lanes' tiles
      int bit = (j - jb) >> csh;
      unsigned m = um >> bit;
      if (m == 0u) break;
      int ahead = __ffs(m) - 1;
      if (ahead > 0) {
        j = jb + ((bit + ahead) << csh);
        continue;
      }
      float4 b = __ldg(&S.rec_box[j]);
      bool test = live && j >= skip_to && lp.x >= b.x && lp.x <= b.z && lp.y >= b.y && lp.y <= b.w;
      if (__any_sync(full, test)) {
        int4 a = __ldg(&S.rec_a[j]), c = __ldg(&S.rec_b[j]);
        float r = __ldg(&S.rec_r[j]);
        int s = a.y;
        if (test && s != cs) {  // the lane enters the next shape: its jobs start here
          cs = s;
          slo = njobs;
          mark = is_eq && s == eq->shape;
        }
        int f = 0;
        if (a.x < 0) {
          if (test) f = within_shape(S, s, lp, r) ? 1 : 0;
        } else if (test) {
          f = within_segment_pre(S, c.x, c.y, c.z, 0, a.z, a.w, a.x, lp, r);  // the lanes' tests run together
          if (f == 2) {
            if (njobs < Q::kJobs) {
              q->job[lane][njobs] = SegJob{s, a.x, lp.x, lp.y, r};
              if (mark) eq_jobs |= 1u << njobs;
              njobs++;
              f = 0;
            } else {
              f = segment_solve(S, c.x, c.y, c.z, a.z, a.w, lp, r);  // queue full: solve now
            }
          }
        }
        if (f == 1) {  // the shape hits
          if (mark) eq_jobs &= (1u << slo) - 1u;
          njobs = slo;  // its queued jobs are moot
          skip_to = c.w;
          if (!is_eq) {
            njobs = glo;
            live = false;
            emit(2 * g + 1, DVG_META_HIT);
            fill(g);
          } else {
            gret = true;
            if (s == eq->shape) eq->hit = 1;
          }
        }
        if (!__any_sync(full, live)) break;
      }
      j++;
    }
    if (live) {  // the group's stroke is decided up to its queued jobs
      if (gret) emit(2 * g + 1, DVG_META_HIT);
      else if (njobs > glo) emit(2 * g + 1, glo | (njobs << 8));
      fill(g);
    }
  }
  return nf;
}


// paint of fragment key (2 * group + is_stroke) at pt
DI float4 frag_color(const DevScene &S, int key, v2 pt) {
  int g = key >> 1;
  return (key & 1) ? paint_color(S, GI(S, g, DVG_GROUP_STROKE_KIND), GI(S, g, DVG_GROUP_STROKE_OFF),
                                 GI(S, g, DVG_GROUP_STROKE_STOPS), pt)
                   : paint_color(S, GI(S, g, DVG_GROUP_FILL_KIND), GI(S, g, DVG_GROUP_FILL_OFF),
                                 GI(S, g, DVG_GROUP_FILL_STOPS), pt);
}

// Blend of a sample's decided candidate fragments (the end of sample_color,
// diffvg.cpp:586-655), fed in group order in one or more runs: the
// fragments that hit (res holds the results of the run's queued segment
// tests) over the background.  With an EdgeQuery the hit flag follows the
// reference's rule: the last fragment that is either of the queried group
// (sets it) or opaque (clears it) decides; without such a fragment the flag
// keeps what the coverage tests of the queried shape set
// (diffvg.cpp:624-633); eq->hit collects those, and eq_jobs marks the
// queried shape's jobs of the run.  With a HitCache, the hit fragment keys
// (blend order) are stored for the backward pass.
struct BlendRun {
  float4 acc;
  int nhit;
  int ev;     // edge-query decision of the last deciding fragment (-1: none)
  int chunk;  // cache chunk taking the keys past the slots (-1: none yet; <= -2: none was left for
              // the key of hit -2 - chunk)
};
DI BlendRun blend_start(const float4 *bg) { return BlendRun{bg ? *bg : F4(0, 0, 0, 0), 0, -1, -1}; }

// Sample idx's entry of the forward pass's fragment cache: its hit keys in
// DVG_HIT_SLOTS slots ([slot][n]), the rest in chunks of DVG_HIT_CHUNK keys
// linked from first[idx], and its key count in cnt[idx] (DVG_HIT_NONE: not
// cached, when the chunks ran out).
struct HitCache {
  int *keys;
  int *chunks;  // [cap][DVG_HIT_CHUNK + 1]: keys, next chunk
  int *first;
  int *count;   // chunks handed out in this pass
  unsigned short *cnt;
  int cap, n, idx;
  DI int key(int i, const int *cid) const {
    return i < DVG_HIT_SLOTS ? __ldg(&keys[(size_t)i * n + idx])
                             : __ldg(&chunks[(size_t)cid[(i - DVG_HIT_SLOTS) / DVG_HIT_CHUNK] * (DVG_HIT_CHUNK + 1) +
                                             (i - DVG_HIT_SLOTS) % DVG_HIT_CHUNK]);
  }
};

DI void cache_key(const HitCache &hc, BlendRun &st, int key) {
  int k = st.nhit;
  if (k < DVG_HIT_SLOTS) {
    hc.keys[(size_t)k * hc.n + hc.idx] = key;
    return;
  }
  if (st.chunk <= -2) return;
  int j = (k - DVG_HIT_SLOTS) % DVG_HIT_CHUNK;
  if (j == 0) {
    int c = hc.chunks ? atomicAdd(hc.count, 1) : hc.cap;
    if (c >= hc.cap) {
      st.chunk = -2 - k;
      return;
    }
    if (k == DVG_HIT_SLOTS) hc.first[hc.idx] = c;
    else hc.chunks[(size_t)st.chunk * (DVG_HIT_CHUNK + 1) + DVG_HIT_CHUNK] = c;
    st.chunk = c;
  }
  hc.chunks[(size_t)st.chunk * (DVG_HIT_CHUNK + 1) + j] = key;
}

template <class Get>
DI void blend_run(const DevScene &S, BlendRun &st, v2 pt, EdgeQ *eq, const Get &get, int nf, unsigned res,
                  unsigned eq_jobs, const HitCache *hc = nullptr) {
  if (eq && (res & eq_jobs)) eq->hit = 1;
  #pragma unroll 1
  for (int i = 0; i < nf; i++) {
    FragRef fr = get(i);
    if (!frag_hit(fr.meta, res)) continue;
    float4 c = frag_color(S, fr.key, pt);
    if (eq) st.ev = (eq->group == (fr.key >> 1)) ? 1 : (c.w >= 1.f ? 0 : st.ev);
    blend(st.acc, c);
    if (hc) cache_key(*hc, st, fr.key);
    st.nhit++;
  }
}

// colour of a finished run; the cache (if set) receives the key count.  A
// sample that found no chunk left adds the further chunks it would have
// taken to the count, so that the count is what the pass needed.
DI float4 blend_finish(const BlendRun &st, const float4 *bg, EdgeQ *eq, const HitCache *hc = nullptr) {
  if (hc) {
    if (st.chunk <= -2) {
      int need = (st.nhit - DVG_HIT_SLOTS + DVG_HIT_CHUNK - 1) / DVG_HIT_CHUNK;
      int asked = (-2 - st.chunk - DVG_HIT_SLOTS) / DVG_HIT_CHUNK + 1;
      if (hc->chunks && need > asked) atomicAdd(hc->count, need - asked);
    }
    hc->cnt[hc->idx] = st.chunk <= -2 ? (unsigned short)DVG_HIT_NONE : (unsigned short)st.nhit;
  }
  if (eq && st.ev >= 0) eq->hit = st.ev;
  if (st.nhit <= 0) return bg ? *bg : F4(0, 0, 0, 0);
  return finish_color(st.acc);
}

// The lane's fragment front blended into st: one out-of-line copy shared by
// the walk's flushes and the final blend, so that the paint and blend code
// is not repeated inside every walk loop.
template <class Front>
static __device__ __noinline__ void blend_front(const DevScene &S, BlendRun &st, v2 pt, EdgeQ *eq, const Front &front,
                                               int nf, unsigned res, unsigned eq_jobs, const HitCache *hc) {
  blend_run(S, st, pt, eq, [&](int i) { return front[i]; }, nf, res, eq_jobs, hc);
}

// State word of a deferred boundary query: its stored fragment count (bits
// 0-7), the blend state of its flushed fragments (bit 28: some hit; bits
// 26-27: edge decision + 1) and its edge hit flag (bit 30).
DI int dq_state(int nf, const BlendRun &st, int hit) {
  return nf | ((st.ev + 1) << 26) | ((st.nhit > 0 ? 1 : 0) << 28) | (hit << 30);
}

// A deferred query's stored candidates, blended over the state its walk
// left (acc: the blend of the fragments it flushed, state: dq_state).
DI float4 blend_deferred(const DevScene &S, const float4 *bg, v2 pt, EdgeQ *eq, const FragRef *frags, int state,
                         float4 acc, unsigned res, unsigned eq_jobs) {
  BlendRun st{acc, (state >> 28) & 1, ((state >> 26) & 3) - 1, -1};
  blend_run(S, st, pt, eq, [&](int i) { return frags[i]; }, state & 0xff, res, eq_jobs);
  return blend_finish(st, bg, eq);
}

// Hands the fp64 walks the warp's fp32 decision left open (npend of them,
// listed by warp_decide) to D's job list, and each owning lane's candidate
// fragments and state to D (dq[qid] = {first fragment, word_y, fp32 results,
// word_w}; dq_col[qid] = acc), when the lists have room; returns whether
// they had (the same in every lane) and sets deferred in the lanes that
// parked.  Without room nothing is stored.
template <class Q, class Front>
DI bool park_open_jobs(const EdgeRecords &D, Q *q, int lane, const Front &front, int nf, bool active,
                       int npend, int qid, int word_y, int word_w, float4 acc, bool &deferred) {
  const unsigned full = 0xffffffffu;
  bool mine = active && ((q->pend_lanes >> lane) & 1u);
  q->qid[lane] = qid;
  // room for the deferring lanes' fragments, then for the warp's jobs
  int nfr = mine ? nf : 0, incl = nfr;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  int fbase = 0, jbase = 0;
  if (lane == 31) fbase = atomicAdd(&D.counts[2], incl);
  fbase = __shfl_sync(full, fbase, 31);
  bool room = (long long)fbase + __shfl_sync(full, incl, 31) <= D.frag_cap;
  if (room) {
    if (lane == 0) jbase = atomicAdd(&D.counts[0], npend);
    jbase = __shfl_sync(full, jbase, 0);
    if ((long long)jbase + npend > D.job_cap) {
      room = false;
      for (int k = jbase + lane; k < D.job_cap && k < jbase + npend; k += 32) D.job_a[k].x = -1;
    }
  }
  __syncwarp();
  if (!room) return false;
  #pragma unroll 1
  for (int k = lane; k < npend; k += 32) {
    int owner, idx;
    SegJob jb = warp_job(q, q->pend[k], owner, idx);
    D.job_a[jbase + k] = make_int4(q->qid[owner], idx, jb.shape, jb.seg);
    D.job_b[jbase + k] = F4(jb.x, jb.y, jb.r, 0.f);
  }
  if (mine) {
    int f0 = fbase + incl - nfr;
    for (int i = 0; i < nf; i++) {
      FragRef fr = front[i];
      D.frag[f0 + i] = make_int2(fr.key, fr.meta);
    }
    D.dq[qid] = make_int4(f0, word_y, (int)q->result[lane], word_w);
    D.dq_res[qid] = 0u;
    D.dq_col[qid] = acc;
    deferred = true;
  }
  __syncwarp();
  return true;
}

// Forward colour of one sample (sample_color, diffvg.cpp:525-655); see
// blend_run for the EdgeQuery rule and the fragment cache.
// Out of line: the boundary pass calls it twice per sample.
// With D (a forward colour pass of 8+ groups), the fp64 walks its fp32
// decision leaves open go to D's job list, as in the boundary pass: the
// lanes that own them park their fragments and blend state under their
// sample number qid, report deferred = true and get their colour from
// k_fwd_finish.
template <class Q>
static __device__ __noinline__ float4 sample_color_fwd(const DevScene &S, const float4 *bg, v2 screen_pt, EdgeQ *eq,
                                                      bool active, Q *q, int lane,
                                                      const HitCache *hc = nullptr,
                                                      const EdgeRecords *D = nullptr, int qid = 0,
                                                      bool *deferred = nullptr) {
  int njobs = 0;
  unsigned eq_jobs = 0;
  bool overflow = false, flushed = false;
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  if (eq) eq->hit = 0;
  BlendRun st = blend_start(bg);
  LocalFront front(q, lane);
  auto flush = [&](int nf, unsigned res, unsigned eqj) { blend_front(S, st, pt, eq, front, nf, res, eqj, hc); };
  int nf = collect_fragments(S, pt, q, front, lane, njobs, eq, eq_jobs, overflow, flushed, active, flush);
  int npend = warp_decide(S, q, lane, njobs);
  bool parked = false;
  if (npend > 0) {
    bool room = D && park_open_jobs(*D, q, lane, front, nf, active, npend, qid,
                                    nf | (st.nhit << 8) | ((overflow ? 1 : 0) << 30), st.chunk, st.acc, parked);
    if (!room) warp_fp64(S, q, lane, npend);
  }
  if (deferred) *deferred = parked;
  if (!active) return F4(0, 0, 0, 0);
  if (overflow) flag_error(S, DVG_EFLAG_CAPACITY);
  if (parked) return F4(0, 0, 0, 0);
  // the final blend in line (the flushes call blend_front)
  blend_run(S, st, pt, eq, [&](int i) { return front[i]; }, nf, q->result[lane], eq_jobs, hc);
  float4 c = blend_finish(st, bg, eq, hc);
  if (hc && overflow) hc->cnt[hc->idx] = DVG_HIT_NONE;
  return c;
}

// One colour query of the paired-lane boundary pass (query qid).  As
// sample_color_fwd, except that the fp64 solves the fp32 decision leaves
// open are handed to E's job list instead of run here, when the lists have
// room: the lanes that own such jobs keep their candidate fragments in
// E.frag, their query state in E.dq[qid] and the blend of the fragments
// their walk already flushed in E.dq_col[qid], and report deferred = true
// (their colour comes from k_edge_finish).  Without room the warp solves its
// jobs in place, as sample_color_fwd does.
template <class Q>
static __device__ __noinline__ float4 sample_color_edge(const DevScene &S, const EdgeRecords &E, const float4 *bg,
                                                       v2 screen_pt, EdgeQ *eq, bool active, Q *q, int lane,
                                                       int qid, bool &deferred) {
  int njobs = 0;
  unsigned eq_jobs = 0;
  bool overflow = false, flushed = false;
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  eq->hit = 0;
  BlendRun st = blend_start(bg);
  LocalFront front(q, lane);
  auto flush = [&](int nf, unsigned res, unsigned eqj) {
    blend_front(S, st, pt, eq, front, nf, res, eqj, nullptr);
  };
  int nf = collect_fragments(S, pt, q, front, lane, njobs, eq, eq_jobs, overflow, flushed, active, flush);
  int npend = warp_decide(S, q, lane, njobs);
  deferred = false;
  if (npend > 0 && !park_open_jobs(E, q, lane, front, nf, active, npend, qid, dq_state(nf, st, eq->hit),
                                   (int)eq_jobs, st.acc, deferred))
    warp_fp64(S, q, lane, npend);
  if (!active) return F4(0, 0, 0, 0);
  if (overflow) flag_error(S, DVG_EFLAG_CAPACITY);
  if (deferred) return F4(0, 0, 0, 0);
  flush(nf, q->result[lane], eq_jobs);  // out of line: the walk kernel's code stays small
  return blend_finish(st, bg, eq);
}

// Adjoint of the blend's output (diffvg.cpp:656-676): d_color of the
// finished colour -> the adjoint at the last fragment; fin receives the
// finished colour of acc.
DI float4 blend_out_adjoint(float4 acc, float4 d_color, float4 &fin) {
  fin = finish_color(acc);
  float4 dc = d_color;
  if (acc.w > 1e-6f) {
    float fa = acc.w;
    float nr = d_color.x / fa, ng = d_color.y / fa, nb = d_color.z / fa;
    dc.w -= (d_color.x * fin.x + d_color.y * fin.y + d_color.z * fin.z) / fa;
    dc.x = nr; dc.y = ng; dc.z = nb;
  }
  return dc;
}

// Reverse step over one fragment (diffvg.cpp:677-698): colour f blended
// onto p; dc is the adjoint after the fragment on entry, before it on exit.
DI void blend_step_adjoint(const DevScene &S, int key, float4 f, float4 p, float4 &dc, v2 pt, float *dp,
                           float *d_tr) {
  float d_pa = dc.w * (1.f - f.w);
  float d_ai = dc.w * (1.f - p.w);
  d_ai += dc.x * (f.x - p.x) + dc.y * (f.y - p.y) + dc.z * (f.z - p.z);
  float d_pr = dc.x * (1 - f.w), d_pg = dc.y * (1 - f.w), d_pb = dc.z * (1 - f.w);
  float4 dci = F4(dc.x * f.w, dc.y * f.w, dc.z * f.w, d_ai);
  int g = key >> 1;
  if (key & 1)
    d_paint_color(S, GI(S, g, DVG_GROUP_STROKE_KIND), GI(S, g, DVG_GROUP_STROKE_OFF),
                  GI(S, g, DVG_GROUP_STROKE_STOPS), pt, dci, dp, d_tr, true);
  else
    d_paint_color(S, GI(S, g, DVG_GROUP_FILL_KIND), GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS), pt,
                  dci, dp, d_tr, true);
  dc = F4(d_pr, d_pg, d_pb, d_pa);
}

// Reverse walk over nh hits in blend order (diffvg.cpp:656-698): key_at(i)
// gives hit i's key, ck[r] the blend state before hit 16 r, and accs[j] the
// state after hit 16 R + j of the last run R (the forward walk leaves them
// there).  Each earlier run's states are rebuilt from its checkpoint with
// the same operations in the same order, so they are the forward walk's
// values.  dc enters as the adjoint of the final blend state and leaves as
// that of the background.
template <class KeyAt>
DI void reverse_hits(const DevScene &S, v2 pt, const KeyAt &key_at, int nh, const float4 *ck, float4 *accs,
                     float4 &dc, float *dp, float *d_tr) {
  int last = (nh - 1) >> 4;
  #pragma unroll 1
  for (int r = last; r >= 0; r--) {
    int lo = r << 4, m = min(nh - lo, 16);
    if (r != last) {
      float4 a = ck[r];
      for (int j = 0; j < m; j++) {
        blend(a, frag_color(S, key_at(lo + j), pt));
        accs[j] = a;
      }
    }
    for (int j = m - 1; j >= 0; j--) {
      int key = key_at(lo + j);
      blend_step_adjoint(S, key, frag_color(S, key, pt), j > 0 ? accs[j - 1] : ck[r], dc, pt, dp, d_tr);
    }
  }
}

// Forward walk over the hits, as reverse_hits expects it: the checkpoint
// before every 16th hit and the states of the current run.
struct HitWalk {
  float4 acc;
  int nh;
  DI void add(const DevScene &S, int key, v2 pt, float4 *ck, float4 *accs) {
    if ((nh & 15) == 0) ck[nh >> 4] = acc;
    blend(acc, frag_color(S, key, pt));
    accs[nh & 15] = acc;
    nh++;
  }
};

// Hits the interior adjoint takes per sample when it collects them itself
// (keys in a small stack array).  A sample with more, and no complete cache
// entry, goes to the deep pass (sample_color_bwd_deep).
#define DVG_BWD_HITS 16

// The hits of the lane's fragment front appended to the walk and to keys
// (deep set past DVG_BWD_HITS); out of line, shared by the walk's flushes
// and the final step.
static __device__ __noinline__ void take_front(const DevScene &S, HitWalk &hw, v2 pt, const SharedFront &front, int nf,
                                              unsigned res, int *keys, float4 *ck, float4 *accs, bool &deep) {
  for (int i = 0; i < nf; i++) {
    FragRef fr = front[i];
    if (!frag_hit(fr.meta, res)) continue;
    if (hw.nh >= DVG_BWD_HITS) {
      deep = true;
      continue;
    }
    keys[hw.nh] = fr.key;
    hw.add(S, fr.key, pt, ck, accs);
  }
}

// Adjoint of sample_color (diffvg.cpp:525-707 with d_color != nullptr).
// d_bg receives the background adjoint with the reference's semantics:
// *assign = 1 when the sample has no fragment (the reference then
// overwrites the pixel's background gradient with d_color).
// cached >= 0: the forward pass's hit fragments of this sample (cached of
// them, keys in hc) stand in for collecting and deciding them again.
// deep is set (and nothing accumulated) when the sample has no cache entry
// and more than DVG_BWD_HITS hits.
DI float4 sample_color_bwd(const DevScene &S, const float4 *bg, v2 screen_pt, float4 d_color, float4 *d_bg,
                           int *assign, float *d_tr, float *dp, bool active, WarpQueue *q, int lane,
                           const HitCache &hc, int cached, bool &deep) {
  int njobs = 0;
  unsigned eq_jobs = 0;
  bool overflow = false, flushed = false;
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  float4 ck[DVG_MAX_FRAGMENTS / 16], accs[16];
  int keys[DVG_BWD_HITS];
  float4 first = bg ? *bg : F4(0, 0, 0, 0);
  HitWalk hw{first, 0};
  deep = false;
  SharedFront front(q, lane);
  auto flush = [&](int nf, unsigned res, unsigned) { take_front(S, hw, pt, front, nf, res, keys, ck, accs, deep); };
  int nf = collect_fragments(S, pt, q, front, lane, njobs, nullptr, eq_jobs, overflow, flushed, active && cached < 0,
                             flush);
  warp_solve(S, q, lane, njobs);
  if (!active) return F4(0, 0, 0, 0);
  if (overflow) {
    flag_error(S, DVG_EFLAG_CAPACITY);
    return F4(0, 0, 0, 0);
  }
  int cid[(DVG_MAX_FRAGMENTS - DVG_HIT_SLOTS) / DVG_HIT_CHUNK];
  if (cached >= 0) {
    for (int i = 0; i < cached; i++) {
      if (i >= DVG_HIT_SLOTS && (i - DVG_HIT_SLOTS) % DVG_HIT_CHUNK == 0) {
        int r = (i - DVG_HIT_SLOTS) / DVG_HIT_CHUNK;
        cid[r] = r == 0 ? __ldg(&hc.first[hc.idx])
                        : __ldg(&hc.chunks[(size_t)cid[r - 1] * (DVG_HIT_CHUNK + 1) + DVG_HIT_CHUNK]);
      }
      hw.add(S, hc.key(i, cid), pt, ck, accs);
    }
  } else {
    flush(nf, q->result[lane], eq_jobs);
  }
  if (deep) return F4(0, 0, 0, 0);
  if (hw.nh <= 0) {
    if (bg) {
      if (d_bg) { *d_bg = d_color; *assign = 1; }
      return *bg;
    }
    return F4(0, 0, 0, 0);
  }
  float4 fin;
  float4 dc = blend_out_adjoint(hw.acc, d_color, fin);
  reverse_hits(S, pt, [&](int i) { return cached >= 0 ? hc.key(i, cid) : keys[i]; }, hw.nh, ck, accs, dc, dp, d_tr);
  if (d_bg) { d_bg->x += dc.x; d_bg->y += dc.y; d_bg->z += dc.z; d_bg->w += dc.w; }
  return fin;
}

// The deep pass's per-warp hit lists: up to DVG_MAX_FRAGMENTS keys per lane
// (key i of lane l in key[i][l]).
struct DeepKeys {
  int key[DVG_MAX_FRAGMENTS][32];
};

// sample_color_bwd for a sample of any depth without a cache entry (the
// deep pass, one warp per block): the hit keys go to the lane's column of
// the warp's DeepKeys.
DI float4 sample_color_bwd_deep(const DevScene &S, const float4 *bg, v2 screen_pt, float4 d_color, float4 *d_bg,
                                int *assign, float *d_tr, float *dp, bool active, WarpQueue *q, DeepKeys *dk,
                                int lane) {
  int njobs = 0;
  unsigned eq_jobs = 0;
  bool overflow = false, flushed = false;
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  float4 ck[DVG_MAX_FRAGMENTS / 16], accs[16];
  float4 first = bg ? *bg : F4(0, 0, 0, 0);
  HitWalk hw{first, 0};
  SharedFront front(q, lane);
  auto flush = [&](int nf, unsigned res, unsigned) {
    for (int i = 0; i < nf; i++) {
      FragRef fr = front[i];
      if (!frag_hit(fr.meta, res)) continue;
      dk->key[hw.nh][lane] = fr.key;
      hw.add(S, fr.key, pt, ck, accs);
    }
  };
  int nf = collect_fragments(S, pt, q, front, lane, njobs, nullptr, eq_jobs, overflow, flushed, active, flush);
  warp_solve(S, q, lane, njobs);
  if (!active) return F4(0, 0, 0, 0);
  if (overflow) {
    flag_error(S, DVG_EFLAG_CAPACITY);
    return F4(0, 0, 0, 0);
  }
  flush(nf, q->result[lane], eq_jobs);
  if (hw.nh <= 0) {
    if (bg) {
      if (d_bg) { *d_bg = d_color; *assign = 1; }
      return *bg;
    }
    return F4(0, 0, 0, 0);
  }
  float4 fin;
  float4 dc = blend_out_adjoint(hw.acc, d_color, fin);
  reverse_hits(S, pt, [&](int i) { return dk->key[i][lane]; }, hw.nh, ck, accs, dc, dp, d_tr);
  if (d_bg) { d_bg->x += dc.x; d_bg->y += dc.y; d_bg->z += dc.z; d_bg->w += dc.w; }
  return fin;
}

// smoothstep / d_smoothstep (diffvg.cpp:817-833)
DI float smoothstep(float d) {
  float t = clampf_((d + 1.f) / 2.f, 0.f, 1.f);
  return t * t * (3 - 2 * t);
}
DI float d_smoothstep(float d, float d_ret) {
  if (d < -1.f || d > 1.f) return 0.f;
  float t = (d + 1.f) / 2.f;
  float d_t = d_ret * (6 * t - 6 * t * t);
  return d_t / 2.f;
}

struct PFrag {
  float4 c;
  int group_stroke;  // 2*group + stroke
  int shape;
  float distance;
  v2 closest;
  PathInfo info;
  int within;
};
static_assert(sizeof(PFrag) <= DVG_PF_BYTES, "prefiltered fragment cache entries");

// Shape-space search radius for a prefiltered stroke's closest point that
// leaves its fragment unchanged.  The coverage smoothstep(|d| + sw) -
// smoothstep(|d| - sw) is exactly 0 once |d| - sw >= 1 in fp32 (both terms
// clamp to 1), so a group whose closest point lies farther than sw_max + 1
// from pt in canvas space gives no fragment.  Under an affine
// canvas-to-shape transform (2x2 part L, corner c8) a canvas distance d is
// at most |L|_F d / |c8| in shape space; the closest-point search keeps the
// same segment and shape whenever the unbounded search's answer lies inside
// the radius, because it only drops candidates that cannot come under it.
// The radius carries a margin for the rounding of both transforms.  Returns
// INFINITY (the unbounded search of compute_distance) for projective or
// ill-conditioned transforms, for groups holding an ellipse (whose distance
// query raises an error), and for groups in which no shape reports a closest
// point (circles, empty paths), where the unbounded search decides the error.
DI float stroke_search_radius(const DevScene &S, int g, v2 pt) {
  const float *c = S.c2s + 9 * g;
  const float *m = S.P + GI(S, g, DVG_GROUP_XFORM_OFF);
  if (c[6] != 0.f || c[7] != 0.f || m[6] != 0.f || m[7] != 0.f) return INFINITY;
  int nsh = GI(S, g, DVG_GROUP_NUM_SHAPES), off = GI(S, g, DVG_GROUP_SHAPES_OFF);
  float sw = 0.f;
  bool reports = false;
  #pragma unroll 1
  for (int k = 0; k < nsh; k++) {
    int s = __ldg(&S.group_shapes[off + k]);
    int kind = SI(S, s, DVG_SHAPE_KIND);
    if (kind == DVG_ELLIPSE) return INFINITY;
    reports |= kind == DVG_RECT || (kind == DVG_PATH && SI(S, s, DVG_SHAPE_NUM_SEGMENTS) > 0);
    sw = fmaxf(sw, stroke_width(S, s));
  }
  if (!reports) return INFINITY;
  float fl = sqrtf(sq(c[0]) + sq(c[1]) + sq(c[3]) + sq(c[4])) / fabsf(c[8]);
  float fm = sqrtf(sq(m[0]) + sq(m[1]) + sq(m[3]) + sq(m[4])) / fabsf(m[8]);
  if (!(fl * fm <= 64.f)) return INFINITY;  // also rejects inf / NaN
  float shift = (fabsf(c[2]) + fabsf(c[5])) / fabsf(c[8]);
  float r = fl * ((sw + 1.f) * 1.01f + 1e-4f * (absmax2(pt) + 1.f)) + 1e-4f * shift + 1e-3f;
  return r < INFINITY ? r : INFINITY;
}

// Coverage fragments of one group at pt (diffvg.cpp:851-905).  Returns the
// number of fragments written (0..2).
DI int prefilter_group(const DevScene &S, int g, v2 pt, PFrag *out) {
  int n = 0;
  int sk = GI(S, g, DVG_GROUP_STROKE_KIND), fk = GI(S, g, DVG_GROUP_FILL_KIND);
  if (sk != DVG_PAINT_NONE) {
    int ms = -1;
    v2 cp = V2(0, 0);
    PathInfo li = {-1, -1, 0.f};
    float d = INFINITY;
    float lim = stroke_search_radius(S, g, pt);
    group_distance(S, g, pt, lim, &ms, &cp, &li, &d);
    if (ms == -1) {
      // with a finite radius: nothing within reach, so the coverage is 0
      if (lim == INFINITY) flag_error(S, DVG_EFLAG_UNSUPPORTED);  // diffvg.cpp:867 asserts
    } else {
      float sw = stroke_width(S, ms);
      float w = smoothstep(fabsf(d) + sw) - smoothstep(fabsf(d) - sw);
      if (w > 0) {
        float4 c = paint_color(S, sk, GI(S, g, DVG_GROUP_STROKE_OFF), GI(S, g, DVG_GROUP_STROKE_STOPS), pt);
        PFrag &f = out[n++];
        f.c = F4(c.x, c.y, c.z, c.w * w);
        f.group_stroke = 2 * g + 1; f.shape = ms; f.distance = d; f.closest = cp; f.info = li; f.within = 1;
      }
    }
  }
  if (fk != DVG_PAINT_NONE) {
    int ms = -1;
    v2 cp = V2(0, 0);
    PathInfo li = {-1, -1, 0.f};
    float d = INFINITY;
    bool found = group_distance(S, g, pt, 1.f, &ms, &cp, &li, &d);
    bool ins = group_inside(S, g, pt, nullptr);
    if (found || ins) {
      if (!ins) d = -d;
      float w = smoothstep(d);
      if (w > 0) {
        float4 c = paint_color(S, fk, GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS), pt);
        PFrag &f = out[n++];
        f.c = F4(c.x, c.y, c.z, c.w * w);
        f.group_stroke = 2 * g; f.shape = ms; f.distance = d; f.closest = cp; f.info = li; f.within = found ? 1 : 0;
      }
    }
  }
  return n;
}

// Sample idx's entry of the prefiltered fragment cache: its first
// DVG_PF_SLOTS fragments in slots ([slot][n]), the rest in chunks of
// DVG_PF_CHUNK fragments (chunks[c][j]) linked from first[idx] through
// next[c]; cnt[idx] holds the count, with DVG_PF_PARTIAL when only the
// leading groups' fragments are stored (no chunk was left, or the sample
// has more fragments than the reference allows).
#define DVG_PF_PARTIAL 0x80
#define DVG_PF_CHUNKS ((DVG_MAX_PREFILTER_FRAGMENTS - DVG_PF_SLOTS) / DVG_PF_CHUNK)
struct PfCache {
  PFrag *slots;
  PFrag *chunks;  // [cap][DVG_PF_CHUNK]
  int *next;      // [cap]
  int *first;     // [n]
  int *count;     // chunks handed out in this pass
  unsigned short *cnt;
  int cap, n, idx;
  DI PFrag *at(int i, const int *cid) const {
    return i < DVG_PF_SLOTS ? &slots[(size_t)i * n + idx]
                            : &chunks[(size_t)cid[(i - DVG_PF_SLOTS) / DVG_PF_CHUNK] * DVG_PF_CHUNK +
                                      (i - DVG_PF_SLOTS) % DVG_PF_CHUNK];
  }
  // the chunk ids of a cached entry of nc fragments
  DI void chunk_ids(int nc, int *cid) const {
    for (int r = 0; DVG_PF_SLOTS + r * DVG_PF_CHUNK < nc; r++)
      cid[r] = r == 0 ? __ldg(&first[idx]) : __ldg(&next[cid[r - 1]]);
  }
};

// sample_color_prefiltered, forward only (diffvg.cpp:835-960)
// With a cache, the sample's fragments (blend order) are stored for the
// backward pass: all of them, or those of the leading groups that fit whole
// with DVG_PF_PARTIAL set in the count, when no chunk is left for the rest
// (the backward pass then resumes the walk after the last stored group).
DI float4 sample_color_prefiltered_fwd(const DevScene &S, const float4 *bg, v2 screen_pt,
                                       const PfCache *pc = nullptr) {
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  int b, e;
  bool list = cand_range(S, pt, b, e);
  float4 acc = bg ? *bg : F4(0, 0, 0, 0);
  int nf = 0, nc = 0, nchunks = 0, asked = 0;
  int cid[DVG_PF_CHUNKS];
  bool caching = pc != nullptr;
  int G = S.num_groups;
  for (int k = b; k < e; k++) {
    int g = list ? __ldg(&S.tile_list[k]) : k;
    if (G > 1 && !box_in_r(S.g_canvas_box[g], pt, S.g_max_radius[g])) continue;
    PFrag fr[2];
    int m = prefilter_group(S, g, pt, fr);
    if (caching && m > 0) {
      if (nc + m > DVG_MAX_PREFILTER_FRAGMENTS) caching = false;
      // chunks for fragments nc .. nc + m - 1
      while (caching && DVG_PF_SLOTS + nchunks * DVG_PF_CHUNK < nc + m) {
        int c = pc->chunks ? atomicAdd(pc->count, 1) : pc->cap;
        asked++;
        if (c >= pc->cap) {
          caching = false;
        } else {
          if (nchunks == 0) pc->first[pc->idx] = c;
          else pc->next[cid[nchunks - 1]] = c;
          cid[nchunks++] = c;
        }
      }
      if (caching) {
        for (int j = 0; j < m; j++) *pc->at(nc + j, cid) = fr[j];
        nc += m;
      }
    }
    for (int j = 0; j < m; j++) blend(acc, fr[j].c);
    nf += m;
  }
  if (pc) {
    // a sample that found no chunk left adds what it would have taken, so
    // that the pass's count is what it needed
    int need = nf > DVG_PF_SLOTS ? (min(nf, DVG_MAX_PREFILTER_FRAGMENTS) - DVG_PF_SLOTS + DVG_PF_CHUNK - 1) /
                                       DVG_PF_CHUNK : 0;
    if (!caching && pc->chunks && need > asked) atomicAdd(pc->count, need - asked);
    pc->cnt[pc->idx] = (unsigned short)(caching ? nc : (nc | DVG_PF_PARTIAL));
  }
  if (nf > DVG_MAX_PREFILTER_FRAGMENTS) flag_error(S, DVG_EFLAG_CAPACITY);
  if (nf <= 0) return bg ? *bg : F4(0, 0, 0, 0);
  return finish_color(acc);
}

// Reverse step over one prefiltered fragment f blended onto p
// (diffvg.cpp:1040-1105); dc is the adjoint after the fragment on entry,
// before it on exit.
DI void pf_step_adjoint(const DevScene &S, const PFrag &f, float4 p, float4 &dc, v2 pt, float *dp, float *d_tr) {
  float d_pa = dc.w * (1.f - f.c.w);
  float d_ai = dc.w * (1.f - p.w);
  d_ai += dc.x * (f.c.x - p.x) + dc.y * (f.c.y - p.y) + dc.z * (f.c.z - p.z);
  float d_pr = dc.x * (1 - f.c.w), d_pg = dc.y * (1 - f.c.w), d_pb = dc.z * (1 - f.c.w);
  float dcir = dc.x * f.c.w, dcig = dc.y * f.c.w, dcib = dc.z * f.c.w;
  int g = f.group_stroke >> 1;
  if (f.group_stroke & 1) {
    float d = f.distance;
    float sw = stroke_width(S, f.shape);
    float apw = fabsf(d) + sw, amw = fabsf(d) - sw;
    float w = smoothstep(apw) - smoothstep(amw);
    if (w != 0) {
      float d_w = w > 0 ? (f.c.w / w) * d_ai : 0.f;
      d_ai *= w;
      d_paint_color(S, GI(S, g, DVG_GROUP_STROKE_KIND), GI(S, g, DVG_GROUP_STROKE_OFF),
                    GI(S, g, DVG_GROUP_STROKE_STOPS), pt, F4(dcir, dcig, dcib, d_ai), dp, d_tr, true);
      float d_apw = d_smoothstep(apw, d_w);
      float d_amw = -d_smoothstep(amw, d_w);
      float d_d = d_apw + d_amw;
      if (d < 0) d_d = -d_d;
      float d_sw = d_apw - d_amw;
      if (fabsf(d_d) > 1e-10f) d_group_distance(S, g, f.shape, pt, f.closest, f.info, d_d, dp, d_tr);
      gadd(dp, SI(S, f.shape, DVG_SHAPE_STROKE_WIDTH_OFF), d_sw);
    }
  } else {
    float d = f.distance;
    float w = smoothstep(d);
    if (w != 0) {
      float d_w = w > 0 ? (f.c.w / w) * d_ai : 0.f;
      d_ai *= w;
      d_paint_color(S, GI(S, g, DVG_GROUP_FILL_KIND), GI(S, g, DVG_GROUP_FILL_OFF), GI(S, g, DVG_GROUP_FILL_STOPS),
                    pt, F4(dcir, dcig, dcib, d_ai), dp, d_tr, true);
      float d_d = d_smoothstep(d, d_w);
      if (d < 0) d_d = -d_d;
      if (fabsf(d_d) > 1e-10f && f.within) d_group_distance(S, g, f.shape, pt, f.closest, f.info, d_d, dp, d_tr);
    }
  }
  dc = F4(d_pr, d_pg, d_pb, d_pa);
}

// Adjoint of sample_color_prefiltered (diffvg.cpp:960-1113) for a sample
// whose fragments are all in the forward pass's cache (cached = their
// count): the reverse walk reads them in place, rebuilding each earlier run
// of 16 blend states from its checkpoint (the same operations in the same
// order).  Any other sample (no valid cache entry, or only its leading
// groups cached) sets deep and is left to
// sample_color_prefiltered_bwd_deep.
DI float4 sample_color_prefiltered_bwd(const DevScene &S, const float4 *bg, v2 screen_pt, float4 d_color,
                                       float4 *d_bg, int *assign, float *d_tr, float *dp, const PfCache &pc,
                                       int cached, bool &deep) {
  deep = cached < 0 || (cached & DVG_PF_PARTIAL) != 0 || cached > DVG_MAX_PREFILTER_FRAGMENTS;
  if (deep) return F4(0, 0, 0, 0);
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  int nc = cached;
  int cid[DVG_PF_CHUNKS];
  pc.chunk_ids(nc, cid);
  float4 ck[DVG_MAX_PREFILTER_FRAGMENTS / 16], accs[16];
  float4 first = bg ? *bg : F4(0, 0, 0, 0);
  float4 acc = first;
  for (int i = 0; i < nc; i++) {
    if ((i & 15) == 0) ck[i >> 4] = acc;
    blend(acc, pc.at(i, cid)->c);
    accs[i & 15] = acc;
  }
  if (nc <= 0) {
    if (bg) {
      if (d_bg) { *d_bg = d_color; *assign = 1; }
      return *bg;
    }
    return F4(0, 0, 0, 0);
  }
  float4 fin;
  float4 dc = blend_out_adjoint(acc, d_color, fin);
  int last = (nc - 1) >> 4;
  #pragma unroll 1
  for (int r = last; r >= 0; r--) {
    int lo = r << 4, m = min(nc - lo, 16);
    if (r != last) {
      float4 a = ck[r];
      for (int j = 0; j < m; j++) {
        blend(a, pc.at(lo + j, cid)->c);
        accs[j] = a;
      }
    }
    for (int j = m - 1; j >= 0; j--) pf_step_adjoint(S, *pc.at(lo + j, cid), j > 0 ? accs[j - 1] : ck[r], dc, pt, dp, d_tr);
  }
  if (d_bg) { d_bg->x += dc.x; d_bg->y += dc.y; d_bg->z += dc.z; d_bg->w += dc.w; }
  return fin;
}

// The prefiltered adjoint for any sample (the deep pass).  The sample's
// fragments come in units: the cached fragments one by one, then the
// candidate groups after the last cached group (0 to 2 fragments each,
// from prefilter_group).  The forward walk keeps, at the start of every run
// of at least DVG_PF_RUN fragments, the blend state and the unit; the
// reverse walk regenerates each run from its checkpoint (prefilter_group is
// deterministic, so the fragments and blend states are the ones of the
// forward walk) and steps back through it.
#define DVG_PF_RUN 4
#define DVG_PF_RUNS (DVG_MAX_PREFILTER_FRAGMENTS / DVG_PF_RUN)
DI float4 sample_color_prefiltered_bwd_deep(const DevScene &S, const float4 *bg, v2 screen_pt, float4 d_color,
                                            float4 *d_bg, int *assign, float *d_tr, float *dp, const PfCache &pc,
                                            int cached) {
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  int b, e;
  bool list = cand_range(S, pt, b, e);
  const int G = S.num_groups;
  int nc = 0, g_done = -1;
  int cid[DVG_PF_CHUNKS];
  if (cached >= 0) {
    nc = min(cached & ~DVG_PF_PARTIAL, DVG_MAX_PREFILTER_FRAGMENTS);
    pc.chunk_ids(nc, cid);
    if (cached & DVG_PF_PARTIAL) g_done = nc > 0 ? pc.at(nc - 1, cid)->group_stroke >> 1 : -1;
    else e = b;  // every fragment is cached: no group is walked
  }
  const int nunits = nc + (e - b);
  // the fragments of unit u (cached entry u, or candidate b + u - nc)
  auto unit = [&](int u, PFrag *out) -> int {
    if (u < nc) {
      out[0] = *pc.at(u, cid);
      return 1;
    }
    int k = b + (u - nc);
    int g = list ? __ldg(&S.tile_list[k]) : k;
    if (g <= g_done) return 0;  // candidates run in ascending group id
    if (G > 1 && !box_in_r(S.g_canvas_box[g], pt, S.g_max_radius[g])) return 0;
    return prefilter_group(S, g, pt, out);
  };
  float4 ck_acc[DVG_PF_RUNS];
  int ck_unit[DVG_PF_RUNS];
  int nruns = 0, in_run = DVG_PF_RUN, nf = 0;
  float4 first = bg ? *bg : F4(0, 0, 0, 0);
  float4 acc = first;
  bool overflow = false;
  PFrag fr[2];
  #pragma unroll 1
  for (int u = 0; u < nunits; u++) {
    int m = unit(u, fr);
    if (m == 0) continue;
    if (nf + m > DVG_MAX_PREFILTER_FRAGMENTS) { overflow = true; break; }
    if (in_run >= DVG_PF_RUN) {  // a run holds DVG_PF_RUN or DVG_PF_RUN + 1 fragments
      ck_acc[nruns] = acc;
      ck_unit[nruns] = u;
      nruns++;
      in_run = 0;
    }
    for (int j = 0; j < m; j++) blend(acc, fr[j].c);
    nf += m;
    in_run += m;
  }
  if (overflow) {
    flag_error(S, DVG_EFLAG_CAPACITY);
    return F4(0, 0, 0, 0);
  }
  if (nf <= 0) {
    if (bg) {
      if (d_bg) { *d_bg = d_color; *assign = 1; }
      return *bg;
    }
    return F4(0, 0, 0, 0);
  }
  float4 fin;
  float4 dc = blend_out_adjoint(acc, d_color, fin);
  PFrag run[DVG_PF_RUN + 1];
  float4 run_acc[DVG_PF_RUN + 1];
  #pragma unroll 1
  for (int r = nruns - 1; r >= 0; r--) {
    int u1 = r + 1 < nruns ? ck_unit[r + 1] : nunits;
    float4 a = ck_acc[r];
    int m = 0;
    #pragma unroll 1
    for (int u = ck_unit[r]; u < u1 && m < DVG_PF_RUN + 1; u++) {
      int k = unit(u, fr);
      for (int j = 0; j < k && m < DVG_PF_RUN + 1; j++) {
        run[m] = fr[j];
        blend(a, fr[j].c);
        run_acc[m] = a;
        m++;
      }
    }
    for (int i = m - 1; i >= 0; i--) pf_step_adjoint(S, run[i], i > 0 ? run_acc[i - 1] : ck_acc[r], dc, pt, dp, d_tr);
  }
  if (d_bg) { d_bg->x += dc.x; d_bg->y += dc.y; d_bg->z += dc.z; d_bg->w += dc.w; }
  return fin;
}

// sample_distance (diffvg.cpp:709-775): signed distance to the closest
// group boundary, negative inside a filled group.
DI float sample_distance(const DevScene &S, v2 screen_pt, float weight, const float *d_dist, float *d_tr, float *dp) {
  v2 pt = V2(screen_pt.x * S.W, screen_pt.y * S.H);
  int min_g = -1, min_s = -1;
  float min_d = 0.f;
  v2 cpt = V2(0, 0);
  PathInfo minfo = {-1, -1, 0.f};
  for (int g = S.num_groups - 1; g >= 0; g--) {
    int s = -1;
    v2 p = V2(0, 0);
    PathInfo li = {-1, -1, 0.f};
    float d = INFINITY;
    if (group_distance(S, g, pt, INFINITY, &s, &p, &li, &d)) {
      if (min_g == -1 || d < min_d) { min_d = d; min_g = g; min_s = s; cpt = p; minfo = li; }
    }
  }
  if (min_g == -1) return min_d;
  min_d *= weight;
  bool ins = false;
  if (GI(S, min_g, DVG_GROUP_FILL_KIND) != DVG_PAINT_NONE) {
    ins = group_inside(S, min_g, pt, nullptr);
    if (ins) min_d = -min_d;
  }
  if (d_dist) {
    float d_abs = ins ? -(*d_dist) : (*d_dist);
    d_group_distance(S, min_g, min_s, pt, cpt, minfo, d_abs, dp, d_tr);
  }
  return min_d;
}
