// Render kernels of the GB300 path: weight image, per-sample colour,
// filtered resolve, interior adjoint, boundary (edge-sampling) adjoint and
// the signed-distance output.
//
// Work decomposition.  Colour kernels run spp CTAs of 256 threads per 16x16
// image tile; the tile's samples are numbered pixel-major with the pixels in
// Morton order, so a warp holds all sub-samples of a compact pixel block
// (4x2 pixels at 2x2 spp, 8x4 at 1 spp) and shares its candidate list.  Sample colours go to a
// per-sample buffer and are filtered by a gather pass per pixel (the
// reference splats them with float atomics, diffvg.cpp:1218-1249); the
// image is written once, atomic-free and deterministic.  The boundary pass
// runs one or two threads per boundary sample (diffvg.cpp:1325-1475).
#include "dvg_internal.h"
#include "dvg_sample.cuh"

#include <atomic>
#include <mutex>

// resident blocks per SM the sample kernels are compiled for (sets their
// register budget: 65536 / (256 * blocks))
#ifndef DVG_SAMPLE_MIN_BLOCKS
#define DVG_SAMPLE_MIN_BLOCKS 2
#endif
// Threads per block (256 k: k groups of 256 samples) of the sample passes and
// of the paired-lane boundary pass; blocks of 512 run one per SM, of 256 two
// (128 registers per thread either way).  One block of 16 warps keeps an SM's
// warps on neighbouring samples, which walk the same candidates and code:
// measured on the stroke-heavy 512x512 workload, forward 4.24 -> 3.76 ms and
// boundary walk 12.87 -> 11.43 ms against two blocks of 256 (blocks of 128 or
// 192 threads were slower still); the prefiltered adjoint (two tiles a block)
// 2.72 -> 2.49 ms on the fill-heavy 1024x1024 workload; the prefiltered
// forward and the sampled interior adjoint measured no better with 512.
#ifndef DVG_FWD_THREADS
#define DVG_FWD_THREADS 512
#endif
static_assert(DVG_FWD_THREADS % 256 == 0 && DVG_FWD_THREADS <= 512, "the forward pass runs 256-sample groups");
#ifndef DVG_BWD_THREADS
#define DVG_BWD_THREADS 256
#endif
#ifndef DVG_PF_FWD_THREADS
#define DVG_PF_FWD_THREADS 256
#endif
#ifndef DVG_PF_BWD_THREADS
#define DVG_PF_BWD_THREADS 512
#endif
static_assert(DVG_BWD_THREADS % 256 == 0 && DVG_BWD_THREADS <= 512 && DVG_PF_FWD_THREADS % 256 == 0 &&
                  DVG_PF_FWD_THREADS <= 512 && DVG_PF_BWD_THREADS % 256 == 0 && DVG_PF_BWD_THREADS <= 512,
              "the sample passes run 256-sample groups");
// resident blocks per SM for a 128-register budget
#define DVG_BLOCKS_FOR(threads) (512 / (threads))
// Resident blocks per SM of the prefiltered forward (its register budget).
// Its per-sample closest-point code is large and fp64-heavy; 16 warps an SM
// left instruction-fetch misses and fp64 latency uncovered, so it runs at
// full occupancy, 8 blocks of 256 with 32 registers, and pays in spills:
// fill-heavy prefiltered 1024x1024 forward 7.28 -> 5.35 ms (4 blocks, 64
// registers: 6.55 ms).  The prefiltered adjoint measured no gain from it.
#ifndef DVG_PF_FWD_BLOCKS
#define DVG_PF_FWD_BLOCKS 8
#endif
#ifndef DVG_FWD_BLOCKS
#define DVG_FWD_BLOCKS DVG_BLOCKS_FOR(DVG_FWD_THREADS)
#endif
// The sampled forward of fill-heavy scenes (64 or more groups, a quarter or
// less stroked) runs two blocks of 512 per SM with 64 registers: its walks are
// short winding-number loops that gain from the extra warps (fill-heavy
// 1024x1024 forward 6.97 -> 6.11 ms), where the stroke walks lose (3.48 ->
// 4.25 ms on the stroke-heavy 512x512 workload).
#ifndef DVG_FWD_FILL_BLOCKS
#define DVG_FWD_FILL_BLOCKS (2 * DVG_FWD_BLOCKS)
#endif
#ifndef DVG_PF_BWD_BLOCKS
#define DVG_PF_BWD_BLOCKS DVG_BLOCKS_FOR(DVG_PF_BWD_THREADS)
#endif
#ifndef DVG_EDGE_THREADS
#define DVG_EDGE_THREADS 512
#endif
#ifndef DVG_EDGE_MIN_BLOCKS
#define DVG_EDGE_MIN_BLOCKS 1
#endif
static_assert(DVG_EDGE_THREADS % 32 == 0 && DVG_EDGE_THREADS <= 512, "the boundary pass runs whole warps, 16 at most");
// the single-lane boundary pass (few groups) keeps two blocks of 256: its walks are short
#define DVG_EDGE1_THREADS 256

namespace dvg {

// The warp queues of the 256-thread sample kernels (8 x sizeof(WarpQueue),
// about 76 KB) are dynamic shared memory: a block may declare at most 48 KB
// statically.
extern __shared__ __align__(16) unsigned char dvg_smem[];
constexpr int kQueueBytes = 8 * (int)sizeof(WarpQueue);
__device__ __forceinline__ WarpQueue *warp_queue() { return reinterpret_cast<WarpQueue *>(dvg_smem) + (threadIdx.x >> 5); }
// the queue of a kernel whose lanes keep their fragment fronts themselves
// (the forward and boundary walks): it stops before the shared front
template <class Q>
__device__ __forceinline__ Q *warp_queue_local() {
  return reinterpret_cast<Q *>(dvg_smem + (threadIdx.x >> 5) * queue_local_bytes<Q>());
}

// Kernels that accumulate into caller-visible outputs do nothing when the
// tile lists overflowed their capacity; the host then grows the lists and
// runs the call again, so nothing is counted twice.
__device__ __forceinline__ bool bins_overflowed(const DevScene &S) {
  return (*(volatile const unsigned *)S.err & DVG_EFLAG_BIN_OVERFLOW) != 0u;
}

// Filter radius and support read from the parameter arena on the device, so
// that no call waits for a host read of a parameter.
__device__ __forceinline__ DevRender load_filter(const DevRender &R0, const DevScene *S) {
  DevRender R = R0;
  float fr = __ldg(R0.fr_ptr);
  bool ok = fr >= 0.f && fr <= 64.f;
  if (!ok && S && threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0) atomicOr(S->err, (unsigned)DVG_EFLAG_FILTER);
  R.fr = ok ? fr : 0.f;
  R.ri = ok ? (int)ceilf(fr) : 0;
  return R;
}

// weight image (weight_kernel, diffvg.cpp:1115-1158), gathered per pixel.
// The reference never passes use_prefiltering to it (diffvg.cpp:1525-1533),
// so the weights always use the jittered positions.
__global__ void __launch_bounds__(256) k_weight(DevRender R0, const __grid_constant__ DevScene S) {
  DevRender R = load_filter(R0, &S);
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= R.w * R.h) return;
  int px = p % R.w, py = p / R.w;
  float ws = 0.f;
  for (int ny = py - R.ri; ny <= py + R.ri; ny++) {
    if (ny < 0 || ny >= R.h) continue;
    for (int nx = px - R.ri; nx <= px + R.ri; nx++) {
      if (nx < 0 || nx >= R.w) continue;
      for (int k = 0; k < R.spp; k++) {
        int idx = (ny * R.w + nx) * R.spp + k, x, y;
        v2 pt = sample_pos(R, idx, false, x, y);
        ws += filter_weight(R.ftype, R.fr, (px + 0.5f) - pt.x, (py + 0.5f) - pt.y);
      }
    }
  }
  R.weight[p] = ws;
}

// sample idx's entry of R's fragment cache
__device__ __forceinline__ HitCache hit_cache(const DevRender &R, int idx) {
  return HitCache{R.hit_keys, R.hit_chunks, R.hit_first, R.hit_chunk_count, R.hit_cnt, R.hit_chunk_cap,
                  R.w * R.h * R.spp, idx};
}
__device__ __forceinline__ PfCache pf_cache(const DevRender &R, int idx) {
  return PfCache{static_cast<PFrag *>(R.pf_frags), static_cast<PFrag *>(R.pf_chunk_frags), R.hit_chunks, R.hit_first,
                 R.hit_chunk_count, R.hit_cnt, R.hit_chunk_cap, R.w * R.h * R.spp, idx};
}

// Sample of thread threadIdx.x in CTA blockIdx.y of its tile: the tile's
// 256 * spp samples are numbered pixel-major, pixels in Morton order, so the
// lanes of a warp hold neighbouring samples and meet the same segments.
__device__ __forceinline__ int morton_x(int k) { return (k & 1) | ((k >> 1) & 2) | ((k >> 2) & 4) | ((k >> 3) & 8); }
__device__ __forceinline__ int morton_y(int k) { return ((k >> 1) & 1) | ((k >> 2) & 2) | ((k >> 3) & 4) | ((k >> 4) & 8); }
__device__ __forceinline__ void tile_sample(int spp, int cta_y, int tid, int &dx, int &dy, int &sub) {
  int j = cta_y * 256 + tid;
  int k = j / spp;
  sub = j - k * spp;
  dx = morton_x(k);
  dy = morton_y(k);
}

// The 256-sample groups of a block of the sample passes (blockDim.x / 256 of
// them): groups of one tile when the tile has that many (blockIdx.y picks
// which), else the groups of neighbouring tiles (blockIdx.x picks which).
// false for a warp whose group lies past the image (it leaves whole).
__device__ __forceinline__ bool block_group(const DevRender &R, int &tile, int &cy) {
  int k = blockDim.x >> 8, sub = threadIdx.x >> 8;
  if (R.spp >= k) {
    tile = blockIdx.x;
    cy = blockIdx.y * k + sub;
    return cy < R.spp;
  }
  int tiles = ((R.w + DVG_TILE - 1) / DVG_TILE) * ((R.h + DVG_TILE - 1) / DVG_TILE);
  tile = blockIdx.x * k + sub;
  cy = blockIdx.y;
  return tile < tiles;
}

// One sample of the forward sample pass: thread tid of the 256-thread group
// cta_y of image tile `tile` (a warp's lanes call it together).
template <bool PREFILTER, class Q>
__device__ __forceinline__ void sample_fwd_one(const DevScene &S, const DevRender &R, int tile, int cta_y, int tid,
                                               float4 *samples, Q *q, int lane,
                                               const EdgeRecords *D = nullptr) {
  int tiles_x = (R.w + DVG_TILE - 1) / DVG_TILE;
  int tx = tile % tiles_x, ty = tile / tiles_x;
  int dx, dy, sub;
  tile_sample(R.spp, cta_y, tid, dx, dy, sub);
  int px = tx * DVG_TILE + dx, py = ty * DVG_TILE + dy;
  bool active = px < R.w && py < R.h;
  if (PREFILTER && !active) return;
  int idx = active ? (py * R.w + px) * R.spp + sub : 0;
  int x, y;
  v2 pt = sample_pos(R, idx, PREFILTER, x, y);
  v2 npt = V2(pt.x / R.w, pt.y / R.h);
  const float4 *bg = R.background ? reinterpret_cast<const float4 *>(R.background) + (y * R.w + x) : nullptr;
  float4 c;
  if (PREFILTER) {
    bool cache = R.pf_frags && !bins_overflowed(S);
    if (R.hit_cnt && !cache) R.hit_cnt[idx] = DVG_HIT_NONE;
    PfCache pc = pf_cache(R, idx);
    c = sample_color_prefiltered_fwd(S, bg, npt, cache ? &pc : nullptr);
  }
  else {
    bool cache = active && R.hit_keys && !bins_overflowed(S);
    if (active && R.hit_cnt && !cache) R.hit_cnt[idx] = DVG_HIT_NONE;
    HitCache hc = hit_cache(R, idx);
    bool parked = false;
    c = sample_color_fwd(S, bg, npt, nullptr, active, q, lane, cache ? &hc : nullptr, D, idx, &parked);
    if (parked) {  // k_fwd_finish writes its colour
      D->ds[atomicAdd(&D->counts[3], 1)] = idx;
      return;
    }
  }
  if (active) samples[idx] = c;
}

// A block of 256 k threads runs groups k blockIdx.y .. k blockIdx.y + k - 1
// of its tile's 256-sample groups (whole warps leave when their group is past
// the tile's spp groups); launch_sample_fwd uses blocks of 256 when a tile
// has fewer samples than a block.
template <bool PREFILTER, class Q, int BLOCKS = DVG_FWD_BLOCKS>
__global__ void __launch_bounds__(PREFILTER ? DVG_PF_FWD_THREADS : DVG_FWD_THREADS,
                                  PREFILTER ? DVG_PF_FWD_BLOCKS : BLOCKS)
    k_sample_fwd(const __grid_constant__ DevScene S, const __grid_constant__ DevRender R, float4 *samples,
                 const __grid_constant__ EdgeRecords D) {
  int cy = blockIdx.y * (blockDim.x >> 8) + (threadIdx.x >> 8);
  if (cy >= R.spp) return;
  sample_fwd_one<PREFILTER>(S, R, blockIdx.x, cy, threadIdx.x & 255, samples, warp_queue_local<Q>(),
                            threadIdx.x & 31, D.job_a ? &D : nullptr);
}

// The samples the forward pass deferred (D.ds): blend each one's parked
// fragments with its fp32 and fp64 results over the blend state it parked,
// continue its fragment-cache entry, write its colour.
__global__ void __launch_bounds__(256) k_fwd_finish(const __grid_constant__ DevScene S,
                                                    const __grid_constant__ DevRender R,
                                                    const __grid_constant__ EdgeRecords D, float4 *samples) {
  int n = *(volatile const int *)&D.counts[3];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int idx = D.ds[k];
    int4 rec = D.dq[idx];
    int x, y;
    v2 spt = sample_pos(R, idx, false, x, y);
    v2 pt = V2(spt.x / R.w * S.W, spt.y / R.h * S.H);
    const float4 *bg = R.background ? reinterpret_cast<const float4 *>(R.background) + (y * R.w + x) : nullptr;
    BlendRun st{D.dq_col[idx], (rec.y >> 8) & 0x3fffff, -1, rec.w};
    bool overflow = (rec.y >> 30) & 1;
    HitCache hc = hit_cache(R, idx);
    const HitCache *hcp = R.hit_keys && !bins_overflowed(S) ? &hc : nullptr;
    const FragRef *frags = reinterpret_cast<const FragRef *>(D.frag + rec.x);
    blend_run(S, st, pt, nullptr, [&](int i) { return frags[i]; }, rec.y & 0xff, (unsigned)rec.z | D.dq_res[idx], 0u,
              hcp);
    float4 c = blend_finish(st, bg, nullptr, hcp);
    if (hcp && overflow) hc.cnt[idx] = DVG_HIT_NONE;
    samples[idx] = c;
  }
}

// filtered pixel colour from the sample colours around it
__global__ void __launch_bounds__(256) k_resolve(DevRender R0, const float4 *samples, float *image) {
  DevRender R = load_filter(R0, nullptr);
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= R.w * R.h) return;
  int px = p % R.w, py = p / R.w;
  float ws = R.weight[p];
  float4 acc = F4(0, 0, 0, 0);
  if (ws > 0) {
    for (int ny = py - R.ri; ny <= py + R.ri; ny++) {
      if (ny < 0 || ny >= R.h) continue;
      for (int nx = px - R.ri; nx <= px + R.ri; nx++) {
        if (nx < 0 || nx >= R.w) continue;
        for (int k = 0; k < R.spp; k++) {
          int idx = (ny * R.w + nx) * R.spp + k, x, y;
          v2 pt = sample_pos(R, idx, R.prefilter != 0, x, y);
          float fw = filter_weight(R.ftype, R.fr, (px + 0.5f) - pt.x, (py + 0.5f) - pt.y);
          float4 c = samples[idx];
          acc = add4(acc, F4(fw * c.x / ws, fw * c.y / ws, fw * c.z / ws, fw * c.w / ws));
        }
      }
    }
  }
  reinterpret_cast<float4 *>(image)[p] = acc;
}

// warp total in lane 0; no block barrier, so a warp that finishes its
// samples early leaves the SM to other blocks instead of waiting for the
// slowest warp of its tile
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// The end of one sample's interior adjoint: its background adjoint and its
// share of the filter-radius adjoint (diffvg.cpp:1250-1268).
__device__ __forceinline__ float sample_bwd_tail(const DevRender &R, int idx, int x, int y, v2 pt, float4 color,
                                                 float4 dbg, int assign, float4 *dbg_val, int *dbg_flag) {
  if (R.d_background) { dbg_val[idx] = dbg; dbg_flag[idx] = assign; }
  float dfr = 0.f;
  for (int dy = -R.ri; dy <= R.ri; dy++)
    for (int dx = -R.ri; dx <= R.ri; dx++) {
      int xx = x + dx, yy = y + dy;
      if (xx >= 0 && xx < R.w && yy >= 0 && yy < R.h && R.weight[yy * R.w + xx] > 0) {
        float ws = R.weight[yy * R.w + xx];
        float xc = xx + 0.5f, yc = yy + 0.5f;
        float fw = filter_weight(R.ftype, R.fr, xc - pt.x, yc - pt.y);
        float4 di = __ldg(reinterpret_cast<const float4 *>(R.d_image) + (yy * R.w + xx));
        float dd = dot4(di, color);
        float d_weight = (dd * ws - fw * dd * (ws - fw)) / (ws * ws);
        dfr += d_filter_weight(R.ftype, R.fr, xc - pt.x, yc - pt.y, d_weight);
      }
    }
  return dfr;
}

// fragment-cache count of sample idx for the backward pass (-1: none valid)
__device__ __forceinline__ int cached_count(const DevRender &R, int idx, bool prefilter) {
  if ((prefilter ? R.pf_frags : (void *)R.hit_keys) && R.hit_cnt && *R.hit_stale == 0u) {
    int c = R.hit_cnt[idx];
    if (c != DVG_HIT_NONE) return c;
  }
  return -1;
}

// One sample of the interior adjoint (render_kernel with d_render_image,
// diffvg.cpp:1160-1268): thread tid of the 256-thread group cta_y of image
// tile `tile`; R carries the filter loaded by load_filter.  A warp's lanes
// call it together (the filter-radius adjoint is summed per warp).  A
// sample deeper than the per-thread lists hold is appended to R.deep_list
// and left to the deep pass (k_sample_bwd_deep).
template <bool PREFILTER>
__device__ __forceinline__ void sample_bwd_one(const DevScene &S, const DevRender &R, int tile, int cta_y, int tid,
                                               float4 *dbg_val, int *dbg_flag, WarpQueue *q, int lane) {
  int tiles_x = (R.w + DVG_TILE - 1) / DVG_TILE;
  int tx = tile % tiles_x, ty = tile / tiles_x;
  int dx, dy, sub;
  tile_sample(R.spp, cta_y, tid, dx, dy, sub);
  int px = tx * DVG_TILE + dx, py = ty * DVG_TILE + dy;
  bool active = px < R.w && py < R.h && !bins_overflowed(S);
  float dfr = 0.f;
  int idx = active ? (py * R.w + px) * R.spp + sub : 0;
  int x, y;
  v2 pt = sample_pos(R, idx, PREFILTER, x, y);
  v2 npt = V2(pt.x / R.w, pt.y / R.h);
  float4 d_color = active ? gather_d_color(R, pt) : F4(0, 0, 0, 0);
  const float4 *bg = R.background ? reinterpret_cast<const float4 *>(R.background) + (y * R.w + x) : nullptr;
  float4 dbg = F4(0, 0, 0, 0);
  int assign = 0;
  float *d_tr = R.d_translation ? R.d_translation + 2 * (y * R.w + x) : nullptr;
  float4 *dbgp = R.d_background ? &dbg : nullptr;
  float4 color;
  bool deep = false;
  if (PREFILTER) {
    color = active ? sample_color_prefiltered_bwd(S, bg, npt, d_color, dbgp, &assign, d_tr, R.d_params,
                                                  pf_cache(R, idx), cached_count(R, idx, true), deep)
                   : F4(0, 0, 0, 0);
  } else {
    color = sample_color_bwd(S, bg, npt, d_color, dbgp, &assign, d_tr, R.d_params, active, q, lane, hit_cache(R, idx),
                             active ? cached_count(R, idx, false) : -1, deep);
  }
  if (active && deep) R.deep_list[atomicAdd(R.deep_count, 1)] = idx;
  else if (active) dfr = sample_bwd_tail(R, idx, x, y, pt, color, dbg, assign, dbg_val, dbg_flag);
  float tot = warp_sum(dfr);
  if (lane == 0 && tot != 0.f) atomicAdd(R.d_params + R.filter_radius_off, tot);
}

template <bool PREFILTER>
__global__ void __launch_bounds__(PREFILTER ? DVG_PF_BWD_THREADS : DVG_BWD_THREADS,
                                  PREFILTER ? DVG_PF_BWD_BLOCKS : DVG_BLOCKS_FOR(DVG_BWD_THREADS))
    k_sample_bwd(const __grid_constant__ DevScene S, DevRender R0, float4 *dbg_val, int *dbg_flag) {
  DevRender R = load_filter(R0, nullptr);
  int tile, cy;
  if (!block_group(R, tile, cy)) return;
  sample_bwd_one<PREFILTER>(S, R, tile, cy, threadIdx.x & 255, dbg_val, dbg_flag, warp_queue(), threadIdx.x & 31);
}

// The deep pass: the interior adjoint of the samples that sample_bwd_one
// listed in R.deep_list, 32 listed samples per warp and step.  Without
// prefiltering the blocks are single warps, each with its per-lane hit lists
// (DeepKeys) in shared memory; the prefiltered samples keep their runs in
// registers and run 8 warps per block.
template <bool PREFILTER>
__device__ __forceinline__ void sample_bwd_deep_one(const DevScene &S, const DevRender &R, int idx, bool active,
                                                    float4 *dbg_val, int *dbg_flag, WarpQueue *q, DeepKeys *dk,
                                                    int lane) {
  int x, y;
  v2 pt = sample_pos(R, idx, PREFILTER, x, y);
  v2 npt = V2(pt.x / R.w, pt.y / R.h);
  float4 d_color = active ? gather_d_color(R, pt) : F4(0, 0, 0, 0);
  const float4 *bg = R.background ? reinterpret_cast<const float4 *>(R.background) + (y * R.w + x) : nullptr;
  float4 dbg = F4(0, 0, 0, 0);
  int assign = 0;
  float *d_tr = R.d_translation ? R.d_translation + 2 * (y * R.w + x) : nullptr;
  float4 *dbgp = R.d_background ? &dbg : nullptr;
  float4 color;
  if (PREFILTER) {
    color = active ? sample_color_prefiltered_bwd_deep(S, bg, npt, d_color, dbgp, &assign, d_tr, R.d_params,
                                                       pf_cache(R, idx), cached_count(R, idx, true))
                   : F4(0, 0, 0, 0);
  } else {
    color = sample_color_bwd_deep(S, bg, npt, d_color, dbgp, &assign, d_tr, R.d_params, active, q, dk, lane);
  }
  float dfr = active ? sample_bwd_tail(R, idx, x, y, pt, color, dbg, assign, dbg_val, dbg_flag) : 0.f;
  float tot = warp_sum(dfr);
  if (lane == 0 && tot != 0.f) atomicAdd(R.d_params + R.filter_radius_off, tot);
}

// the listed samples of one scene, from warp `warp` of `nwarps` on
template <bool PREFILTER>
__device__ __forceinline__ void deep_samples(const DevScene &S, const DevRender &R, float4 *dbg_val, int *dbg_flag,
                                             WarpQueue *q, DeepKeys *dk, int warp, int nwarps, int lane) {
  if (bins_overflowed(S)) return;
  int count = *(volatile const int *)R.deep_count;
  #pragma unroll 1
  for (int base = warp * 32; base < count; base += nwarps * 32) {
    int j = base + lane;
    bool act = j < count;
    sample_bwd_deep_one<PREFILTER>(S, R, act ? R.deep_list[j] : 0, act, dbg_val, dbg_flag, q, dk, lane);
  }
}

__global__ void __launch_bounds__(32) k_sample_bwd_deep(const __grid_constant__ DevScene S, DevRender R0,
                                                        float4 *dbg_val, int *dbg_flag) {
  __shared__ WarpQueue wq;
  __shared__ DeepKeys dk;
  DevRender R = load_filter(R0, nullptr);
  deep_samples<false>(S, R, dbg_val, dbg_flag, &wq, &dk, blockIdx.x, gridDim.x, threadIdx.x);
}

__global__ void __launch_bounds__(256) k_sample_bwd_deep_pf(const __grid_constant__ DevScene S, DevRender R0,
                                                            float4 *dbg_val, int *dbg_flag) {
  DevRender R = load_filter(R0, nullptr);
  deep_samples<true>(S, R, dbg_val, dbg_flag, nullptr, nullptr, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                     (gridDim.x * blockDim.x) >> 5, threadIdx.x & 31);
}

// Background adjoint in sample order per pixel: a sample without fragments
// overwrites the pixel's value with its d_color, the others add to it
// (diffvg.cpp:596-604, 699-704).
__global__ void k_bg_combine(const __grid_constant__ DevScene S, DevRender R, const float4 *dbg_val,
                             const int *dbg_flag) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= R.w * R.h || bins_overflowed(S)) return;
  float4 *dst = reinterpret_cast<float4 *>(R.d_background) + p;
  float4 v = *dst;
  for (int k = 0; k < R.spp; k++) {
    int idx = p * R.spp + k;
    float4 c = dbg_val[idx];
    v = dbg_flag[idx] ? c : add4(v, c);
  }
  *dst = v;
}

// Boundary adjoint (sample_boundary_kernel + render_edge_kernel,
// diffvg.cpp:1325-1475) in three passes:
//   k_edge_sample  draws every boundary sample (same pcg streams and CDFs as
//                  the reference) and files it under its canvas tile and
//                  its cell of 4x4 pixels in the tile;
//   k_edge_order   turns the per-cell counts into a cell-sorted order;
//   k_edge_eval    evaluates the two sides of each boundary point in that
//                  order, so that a warp's samples share a candidate list
//                  and mostly the same segment tests.
// The reference sorts its boundary samples by Morton code for the same
// coherence (diffvg.cpp:1594-1599); the order only changes the order of the
// gradient atomics.
__global__ void __launch_bounds__(256) k_edge_sample(const __grid_constant__ DevScene S, DevRender R, EdgeRecords E) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  int n = R.w * R.h * R.spp;
  if (idx >= n) return;
  E.key[idx] = -1;
  if (S.num_total <= 0 || bins_overflowed(S)) return;
  Pcg rng = pcg_init(idx, R.seed);
  float u = pcg_float(rng);
  int sid = cdf_sample(S.smp_cdf, S.num_total, u, nullptr);
  int s = S.smp_shape[sid], g = S.smp_group[sid];
  // diffvg.cpp:1343 indexes the pmf by shape id
  float pmf = s < S.num_total ? S.smp_pmf[s] : 0.f;
  if (pmf <= 0) return;
  float pdf = 0.f;
  v2 normal = V2(0, 0);
  float t = pcg_float(rng);
  BData bd = {0, 0, 0.f, 0};
  v2 lpt = sample_boundary(S, g, s, t, &normal, &pdf, &bd);
  if (pdf <= 0) return;
  int xo = GI(S, g, DVG_GROUP_XFORM_OFF);
  float s2c[9], c2s[9];
#pragma unroll
  for (int i = 0; i < 9; i++) { s2c[i] = pget(S, xo + i); c2s[i] = S.c2s[9 * g + i]; }
  v2 bpt = xform_pt(s2c, lpt);
  normal = xform_normal(c2s, normal);
  bpt.x /= S.W;
  bpt.y /= S.H;
  pdf = pmf * pdf;
  int bx = (int)(bpt.x * R.w), by = (int)(bpt.y * R.h);
  if (bx < 0 || bx >= R.w || by < 0 || by >= R.h) return;
  // canvas tile of the boundary point (clamped into the grid), then its cell
  // inside the tile
  float cx = bpt.x * S.W, cy = bpt.y * S.H;
  int tx = min(max((int)floorf(cx / DVG_TILE), 0), S.tiles_x - 1);
  int ty = min(max((int)floorf(cy / DVG_TILE), 0), S.tiles_y - 1);
  int lx = min(max((int)floorf(cx) - tx * DVG_TILE, 0), DVG_TILE - 1) >> DVG_EDGE_CELL_SHIFT;
  int ly = min(max((int)floorf(cy) - ty * DVG_TILE, 0), DVG_TILE - 1) >> DVG_EDGE_CELL_SHIFT;
  int cell = 0;
  #pragma unroll
  for (int bit = 0; bit < 4; bit++) cell |= (((lx >> bit) & 1) << (2 * bit)) | (((ly >> bit) & 1) << (2 * bit + 1));
  int key = (ty * S.tiles_x + tx) * DVG_EDGE_CELLS + cell;
  E.key[idx] = key;
  E.rank[idx] = atomicAdd(&E.tile_count[key], 1);
  E.a[idx] = F4(bpt.x, bpt.y, normal.x, normal.y);
  E.b[idx] = F4(lpt.x, lpt.y, pdf, t);
  E.c[idx] = make_int4(g, s, bd.base_point_id, bd.point_id);
  E.d[idx] = make_float2(bd.t, (float)bd.is_stroke);
}

// exclusive scan of the per-cell sample counts (one block of 1024 threads)
__global__ void k_edge_scan(const __grid_constant__ DevScene S, EdgeRecords E) {
  int T = S.tiles_x * S.tiles_y * DVG_EDGE_CELLS;
  __shared__ int part[1024];
  int per = (T + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(lo + per, T);
  int sum = 0;
  for (int i = lo; i < hi; i++) sum += E.tile_count[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x > 0 ? part[threadIdx.x - 1] : 0;
  for (int i = lo; i < hi; i++) {
    E.tile_start[i] = run;
    run += E.tile_count[i];
  }
  if (threadIdx.x == 0) E.tile_start[T] = part[blockDim.x - 1];
}

__global__ void k_edge_order(EdgeRecords E, int n) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  int key = E.key[idx];
  if (key >= 0) E.order[E.tile_start[key] + E.rank[idx]] = idx;
}

// The end of render_edge_kernel (diffvg.cpp:1418-1474) for one boundary
// sample whose two colours are known: orient the normal towards the hit
// side, and accumulate the Reynolds-transport contribution.
DI void edge_accumulate(const DevScene &S, const DevRender &R, int g, int s, v2 bpt, v2 normal, v2 lpt, float pdf,
                        float t, const BData &bd, float4 cin, int hin, float4 cout, int hout) {
  if (!hin && !hout) return;
  if (!hin) {
    normal = neg2(normal);
    float4 tmp = cin; cin = cout; cout = tmp;
  }
  int bx = min(max((int)(bpt.x * R.w), 0), R.w - 1), by = min(max((int)(bpt.y * R.h), 0), R.h - 1);
  v2 sbpt = V2(bpt.x * R.w, bpt.y * R.h);
  float4 dc = gather_d_color(R, sbpt);
  float norm = (float)(S.W * S.H);
  dc = F4(dc.x / norm, dc.y / norm, dc.z / norm, dc.w / norm);
  float contrib = dot4(sub4(cin, cout), dc) / pdf;
  accumulate_boundary_gradient(S, g, s, contrib, t, normal, bd, lpt, R.d_params);
  if (R.d_translation) {
    atomicAdd(&R.d_translation[2 * (by * R.w + bx) + 0], normal.x * contrib);
    atomicAdd(&R.d_translation[2 * (by * R.w + bx) + 1], normal.y * contrib);
  }
}

// Boundary samples (render_edge_kernel, diffvg.cpp:1388-1475).  With PAIRS
// set, the two colour queries of a sample (just inside and just outside the
// boundary) run in adjacent lanes: their points are 2e-4 canvas widths apart,
// so the two lanes walk the same candidates and tests, and a warp spreads its
// divergence over 16 samples instead of 32 walked twice; the even lane
// finishes the sample.  The paired pass also hands the fp64 root walks that
// its fp32 decision leaves open to k_edge_jobs (sample_color_edge): a sample
// with such a query is listed in E.ds and finished by k_edge_finish.
// Without PAIRS one lane runs both queries: for scenes of few shapes the
// walks are short and the gradient atomics, aggregated per warp, are what
// costs.
// One lane (gi: index of the lane over the pass) of the boundary pass; R
// carries the filter loaded by load_filter; a warp's lanes call it together.
template <bool PAIRS, class Q>
__device__ __forceinline__ void edge_eval_one(const DevScene &S, const DevRender &R, const EdgeRecords &E, long long gi,
                                              Q *q, int lane) {
  const unsigned full = 0xffffffffu;
  int i = (int)(PAIRS ? gi >> 1 : gi);
  bool outside = PAIRS && (gi & 1);
  int T = S.tiles_x * S.tiles_y * DVG_EDGE_CELLS;
  bool active = i < E.tile_start[T] && !bins_overflowed(S);
  int idx = active ? E.order[i] : 0;
  float4 a = active ? E.a[idx] : F4(0.5f, 0.5f, 1.f, 0.f), b = active ? E.b[idx] : F4(0, 0, 1, 0);
  int4 c = active ? E.c[idx] : make_int4(0, 0, 0, 0);
  float2 d = active ? E.d[idx] : make_float2(0.f, 0.f);
  v2 bpt = V2(a.x, a.y), normal = V2(a.z, a.w), lpt = V2(b.x, b.y);
  float pdf = b.z, t = b.w;
  int g = c.x, s = c.y;
  BData bd = {c.z, c.w, d.x, d.y != 0.f ? 1 : 0};
  int bx = min(max((int)(bpt.x * R.w), 0), R.w - 1), by = min(max((int)(bpt.y * R.h), 0), R.h - 1);
  EdgeQ qq = {g, s, 0};
  const float4 *bg = R.background ? reinterpret_cast<const float4 *>(R.background) + (by * R.w + bx) : nullptr;
  v2 qpt = outside ? add2(bpt, scl2(1e-4f, normal)) : sub2(bpt, scl2(1e-4f, normal));
  float4 cin, cout;
  int hin, hout;
  if (PAIRS) {
    bool deferred = false;
    if (E.job_a) {
      cin = sample_color_edge(S, E, bg, qpt, &qq, active, q, lane, (int)gi, deferred);
    } else {
      cin = sample_color_fwd(S, bg, qpt, &qq, active, q, lane);
    }
    hin = qq.hit;
    unsigned dm = __ballot_sync(full, deferred);
    cout = F4(__shfl_xor_sync(full, cin.x, 1), __shfl_xor_sync(full, cin.y, 1), __shfl_xor_sync(full, cin.z, 1),
              __shfl_xor_sync(full, cin.w, 1));
    hout = __shfl_xor_sync(full, hin, 1);
    if (!active) return;
    if ((dm >> (lane & ~1)) & 3u) {  // the sample waits for deferred jobs: k_edge_finish completes it
      if (!deferred) {
        E.dq[gi] = make_int4(-1, hin, 0, 0);
        E.dq_col[gi] = cin;
      }
      if (!outside) E.ds[atomicAdd(&E.counts[3], 1)] = i;
      return;
    }
  } else {
    cin = sample_color_fwd(S, bg, qpt, &qq, active, q, lane);
    hin = qq.hit;
    EdgeQ qo = {g, s, 0};
    cout = sample_color_fwd(S, bg, add2(bpt, scl2(1e-4f, normal)), &qo, active, q, lane);
    hout = qo.hit;
  }
  if (outside || !active) return;
  edge_accumulate(S, R, g, s, bpt, normal, lpt, pdf, t, bd, cin, hin, cout, hout);
}

template <bool PAIRS, class Q>
__global__ void __launch_bounds__(PAIRS ? DVG_EDGE_THREADS : DVG_EDGE1_THREADS,
                                  PAIRS ? DVG_EDGE_MIN_BLOCKS : DVG_SAMPLE_MIN_BLOCKS)
    k_edge_eval(const __grid_constant__ DevScene S, DevRender R0, const __grid_constant__ EdgeRecords E) {
  DevRender R = load_filter(R0, nullptr);
  edge_eval_one<PAIRS>(S, R, E, (long long)blockIdx.x * blockDim.x + threadIdx.x, warp_queue_local<Q>(),
                       threadIdx.x & 31);
}

// The deferred fp64 root walks of the paired boundary pass, one per thread
// (full warps): each sets its result bit in its query's dq_res.
// The deferred fp64 root walks, first part (one job per thread): a
// quadratic segment's test whole; for a cubic segment the normalised
// distance quintic (kept in job_q) and its root brackets (quintic_brackets),
// which go to the task list for k_edge_roots.  The brackets of a warp are
// reserved together; when the list has no room the lanes walk their
// brackets here, as segment_root_test does.
__device__ __forceinline__ void edge_jobs_all(const DevScene &S, const EdgeRecords &E) {
  const unsigned full = 0xffffffffu;
  int lane = threadIdx.x & 31;
  int n = min(*(volatile const int *)&E.counts[0], E.job_cap);
  // warp-uniform trip count: the lanes of a warp take jobs k0 .. k0 + 31
  for (int k0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); k0 < n; k0 += gridDim.x * blockDim.x) {
    int k = k0 + lane;
    int4 ja = k < n ? E.job_a[k] : make_int4(-1, 0, 0, 0);
    float lo[5], hi[5];
    int nb = 0, hit = 0;
    Quintic q{};
    CubicSeg c{};
    v2 pt = V2(0.f, 0.f);
    if (ja.x >= 0) {
      float4 jb = E.job_b[k];
      int s = ja.z;
      int po = SI(S, s, DVG_SHAPE_PARAM_OFF), np = SI(S, s, DVG_SHAPE_NUM_POINTS);
      int th = SI(S, s, DVG_SHAPE_THICKNESS_OFF), nc = __ldg(&S.segment_ctrl[ja.w]), i0 = __ldg(&S.seg_point[ja.w]);
      pt = V2(jb.x, jb.y);
      if (nc != 2 || !E.task) {
        hit = segment_root_test(S, po, np, th, nc, i0, pt, jb.z);
      } else {
        c = cubic_seg(S, po, np, th, i0, jb.z);
        q = cubic_quintic(c.p[0], c.p[1], c.p[2], c.p[3], pt);
        nb = quintic_brackets(q, lo, hi);
        double *qk = E.job_q + 5 * (size_t)k;
        qk[0] = q.B;
        qk[1] = q.C;
        qk[2] = q.D;
        qk[3] = q.E;
        qk[4] = q.F;
      }
    }
    int incl = nb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(full, incl, o);
      if (lane >= o) incl += v;
    }
    int total = __shfl_sync(full, incl, 31), base = 0;
    if (lane == 0 && total > 0) base = atomicAdd(&E.counts[4], total);
    base = __shfl_sync(full, base, 0);
    if ((long long)base + total <= E.task_cap) {
      for (int i = 0; i < nb; i++)
        E.task[base + incl - nb + i] = make_int4(k, __float_as_int(lo[i]), __float_as_int(hi[i]), 0);
    } else {
      for (int i = incl - nb; i < incl; i++)  // the reserved slots that fit: none of them is walked
        if (base + i < E.task_cap) E.task[base + i] = make_int4(-1, 0, 0, 0);
      for (int i = 0; i < nb && !hit; i++) hit = cubic_root_hits(c, pt, quintic_root(q, lo[i], hi[i])) ? 1 : 0;
    }
    if (hit) atomicOr(&E.dq_res[ja.x], 1u << ja.y);
  }
}

__global__ void __launch_bounds__(256) k_edge_jobs(const __grid_constant__ DevScene S, const __grid_constant__ EdgeRecords E) {
  edge_jobs_all(S, E);
}

// The deferred fp64 root walks, second part: the safeguarded Newton /
// bisection walk of every root bracket (quintic_root, within_distance.h:
// 251-269), one bracket per lane and one iteration per step; a lane whose
// walk stops runs the stroke test at the root, sets the job's bit when it
// hits, and takes the next bracket of the list, so the lanes of a warp stay
// busy whatever the iteration counts of their brackets.
__device__ __forceinline__ void edge_roots_all(const DevScene &S, const EdgeRecords &E) {
  const unsigned full = 0xffffffffu;
  int lane = threadIdx.x & 31;
  int ntask = min(*(volatile const int *)&E.counts[4], E.task_cap);
  int cur = -1, job = -1, it = 0;  // cur: the lane's bracket (-1: none yet, >= ntask: no more)
  float lb = 0.f, ub = 0.f, t = 0.f;
  Quintic q{};
  #pragma unroll 1
  while (true) {
    unsigned idle = __ballot_sync(full, cur < 0);
    if (idle) {
      int first = 0;
      if (lane == 0) first = atomicAdd(&E.counts[5], __popc(idle));
      first = __shfl_sync(full, first, 0);
      if (cur < 0) {
        cur = first + __popc(idle & ((1u << lane) - 1u));
        if (cur < ntask) {
          int4 tk = E.task[cur];
          if (tk.x < 0) {
            cur = -1;
          } else {
            job = tk.x;
            const double *qk = E.job_q + 5 * (size_t)job;
            q.A = 1.0;
            q.B = qk[0];
            q.C = qk[1];
            q.D = qk[2];
            q.E = qk[3];
            q.F = qk[4];
            lb = __int_as_float(tk.y);
            ub = __int_as_float(tk.z);
            t = 0.5f * (lb + ub);
            it = 0;
          }
        }
      }
    }
    if (__all_sync(full, cur >= ntask)) break;
    if (cur < 0 || cur >= ntask) continue;
    // one iteration of quintic_root
    if (!(t >= lb && t <= ub)) t = 0.5f * (lb + ub);
    double value = quintic_eval(q, t);
    if (!(fabs(value) < 1e-5f || it == 19)) {
      if (value > 0.f) ub = t; else lb = t;
      if (!(lb > ub)) {
        double derivative = quintic_deriv(q, t);
        t = (float)(t - ddiv(value, derivative));
      }
      it++;
      continue;
    }
    // the walk stopped at t: the stroke test there
    int4 ja = E.job_a[job];
    float4 jb = E.job_b[job];
    int s = ja.z;
    CubicSeg c = cubic_seg(S, SI(S, s, DVG_SHAPE_PARAM_OFF), SI(S, s, DVG_SHAPE_NUM_POINTS),
                           SI(S, s, DVG_SHAPE_THICKNESS_OFF), __ldg(&S.seg_point[ja.w]), jb.z);
    if (cubic_root_hits(c, V2(jb.x, jb.y), t)) atomicOr(&E.dq_res[ja.x], 1u << ja.y);
    cur = -1;
  }
}
__global__ void __launch_bounds__(256) k_edge_roots(const __grid_constant__ DevScene S, const __grid_constant__ EdgeRecords E) {
  edge_roots_all(S, E);
}

// Deferred boundary sample k of E.ds: blend each deferred query's fragments
// with its fp32 and fp64 results, take the other query's colour from the
// first pass, and accumulate the sample.
__device__ __forceinline__ void edge_finish_one(const DevScene &S, const DevRender &R, const EdgeRecords &E, int k) {
  int i = E.ds[k];
  int idx = E.order[i];
  float4 a = E.a[idx], b = E.b[idx];
  int4 c = E.c[idx];
  float2 d = E.d[idx];
  v2 bpt = V2(a.x, a.y), normal = V2(a.z, a.w), lpt = V2(b.x, b.y);
  int g = c.x, s = c.y;
  BData bd = {c.z, c.w, d.x, d.y != 0.f ? 1 : 0};
  int bx = min(max((int)(bpt.x * R.w), 0), R.w - 1), by = min(max((int)(bpt.y * R.h), 0), R.h - 1);
  const float4 *bg = R.background ? reinterpret_cast<const float4 *>(R.background) + (by * R.w + bx) : nullptr;
  float4 col[2];
  int hit[2];
  for (int side = 0; side < 2; side++) {
    int qid = 2 * i + side;
    int4 rec = E.dq[qid];
    if (rec.x < 0) {
      col[side] = E.dq_col[qid];
      hit[side] = rec.y;
      continue;
    }
    v2 qpt = side ? add2(bpt, scl2(1e-4f, normal)) : sub2(bpt, scl2(1e-4f, normal));
    EdgeQ eq = {g, s, (rec.y >> 30) & 1};
    unsigned res = (unsigned)rec.z | E.dq_res[qid];
    col[side] = blend_deferred(S, bg, V2(qpt.x * S.W, qpt.y * S.H), &eq,
                               reinterpret_cast<const FragRef *>(E.frag + rec.x), rec.y, E.dq_col[qid], res,
                               (unsigned)rec.w);
    hit[side] = eq.hit;
  }
  edge_accumulate(S, R, g, s, bpt, normal, lpt, b.z, b.w, bd, col[0], hit[0], col[1], hit[1]);
}

__global__ void __launch_bounds__(256) k_edge_finish(const __grid_constant__ DevScene S, DevRender R0,
                                                     const __grid_constant__ EdgeRecords E) {
  DevRender R = load_filter(R0, nullptr);
  int n = *(volatile const int *)&E.counts[3];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) edge_finish_one(S, R, E, k);
}

__global__ void __launch_bounds__(256) k_edge_finish_batch(const BatchScene *B, int nb, const int *order) {
  for (int r = 0; r < nb; r++) {
    const BatchScene &b = B[__ldg(&order[r])];
    if (!b.E.job_a) continue;
    DevRender R = load_filter(b.R, nullptr);
    int n = *(volatile const int *)&b.E.counts[3];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) edge_finish_one(b.S, R, b.E, k);
  }
}

// signed distance output (render_kernel's sdf branch, diffvg.cpp:1273-1293)
__global__ void __launch_bounds__(256) k_sdf(const __grid_constant__ DevScene S, DevRender R,
                                             const float *eval_positions, int num_eval, float *sdf,
                                             const float *d_sdf) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  int n = eval_positions ? num_eval : R.w * R.h * R.spp;
  if (idx >= n || bins_overflowed(S)) return;
  int x, y;
  v2 pt;
  if (eval_positions) {
    pt = V2(eval_positions[2 * idx], eval_positions[2 * idx + 1]);
    x = (int)pt.x;
    y = (int)pt.y;
  } else {
    pt = sample_pos(R, idx, R.prefilter != 0, x, y);
  }
  v2 npt = V2(pt.x / R.w, pt.y / R.h);
  float d_dist = 0.f;
  if (d_sdf) d_dist = eval_positions ? d_sdf[idx] : d_sdf[y * R.w + x];
  float weight = eval_positions ? 1.f : 1.f / R.spp;
  bool in_image = x >= 0 && x < R.w && y >= 0 && y < R.h;
  float *d_tr = (R.d_translation && in_image) ? R.d_translation + 2 * (y * R.w + x) : nullptr;
  float dist = sample_distance(S, npt, weight, d_sdf ? &d_dist : nullptr, d_tr, R.d_params);
  if (sdf) {
    if (eval_positions) sdf[idx] += dist;
    else atomicAdd(&sdf[y * R.w + x], dist);
  }
}

// bitwise comparison of the parameter arena with the forward pass's copy
__global__ void k_hit_check(const float *params, const float *fwd_params, int n, unsigned *stale) {
  const unsigned *a = reinterpret_cast<const unsigned *>(params), *b = reinterpret_cast<const unsigned *>(fwd_params);
  bool diff = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) diff |= a[i] != b[i];
  if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(stale, 1u);
}

// ---------------------------------------------------------------------------
// Persistent batched passes.  One launch serves every scene of a batch: warps
// take work items from a global counter until the batch's items run out, so
// small scenes do not leave the GPU idle between launches and large ones are
// spread over every SM.  An item is `spt` consecutive 32-sample chunks of one
// scene (spt: samples per thread).  Scenes are taken in `order` (largest
// first); item_start[r] is the first item of the r-th scene of that order.

// range r with item_start[r] <= item < item_start[r + 1] (item_start in
// global or shared memory: plain loads)
__device__ __forceinline__ int batch_range_of(const int *item_start, int nb, int item) {
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (item_start[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The next item of the warp (lane 0 takes it, every lane gets it).
__device__ __forceinline__ int batch_next(int *counter, int lane) {
  int item = 0;
  if (lane == 0) item = atomicAdd(counter, 1);
  return __shfl_sync(0xffffffffu, item, 0);
}

// forward sample pass: a scene has tiles * spp * 8 chunks (the 8 warps of a
// tile's 256-sample group)
template <class Q>
__global__ void __launch_bounds__(512, 1)
    k_sample_fwd_batch(const BatchScene *B, int nb, const int *order, const int *item_start, int spt, int *counter) {
  int lane = threadIdx.x & 31;
  Q *q = warp_queue_local<Q>();
  int total = __ldg(&item_start[nb]);
  #pragma unroll 1
  for (int item = batch_next(counter, lane); item < total; item = batch_next(counter, lane)) {
    int r = batch_range_of(item_start, nb, item);
    const BatchScene &b = B[__ldg(&order[r])];
    int spp = b.R.spp, nchunk = ((b.R.w + DVG_TILE - 1) / DVG_TILE) * ((b.R.h + DVG_TILE - 1) / DVG_TILE) * spp * 8;
    int c0 = (item - __ldg(&item_start[r])) * spt;
    #pragma unroll 1
    for (int c = c0; c < c0 + spt && c < nchunk; c++) {
      int rest = c >> 3;
      sample_fwd_one<false>(b.S, b.R, rest / spp, rest % spp, (c & 7) * 32 + lane, b.samples, q, lane);
    }
  }
}

// interior adjoint
__global__ void __launch_bounds__(256, DVG_SAMPLE_MIN_BLOCKS)
    k_sample_bwd_batch(const BatchScene *B, int nb, const int *order, const int *item_start, int spt, int *counter) {
  int lane = threadIdx.x & 31;
  WarpQueue *q = warp_queue();
  int total = __ldg(&item_start[nb]);
  #pragma unroll 1
  for (int item = batch_next(counter, lane); item < total; item = batch_next(counter, lane)) {
    int r = batch_range_of(item_start, nb, item);
    const BatchScene &b = B[__ldg(&order[r])];
    DevRender R = load_filter(b.R, nullptr);
    int spp = R.spp, nchunk = ((R.w + DVG_TILE - 1) / DVG_TILE) * ((R.h + DVG_TILE - 1) / DVG_TILE) * spp * 8;
    int c0 = (item - __ldg(&item_start[r])) * spt;
    #pragma unroll 1
    for (int c = c0; c < c0 + spt && c < nchunk; c++) {
      int rest = c >> 3;
      sample_bwd_one<false>(b.S, R, rest / spp, rest % spp, (c & 7) * 32 + lane, nullptr, nullptr, q, lane);
    }
  }
}

// the deep pass of every scene of the batch (no prefiltering in batches)
__global__ void __launch_bounds__(32) k_sample_bwd_deep_batch(const BatchScene *B, int nb, const int *order) {
  __shared__ WarpQueue wq;
  __shared__ DeepKeys dk;
  for (int r = 0; r < nb; r++) {
    const BatchScene &b = B[__ldg(&order[r])];
    DevRender R = load_filter(b.R, nullptr);
    deep_samples<false>(b.S, R, nullptr, nullptr, &wq, &dk, blockIdx.x, gridDim.x, threadIdx.x);
  }
}

// paired-lane boundary pass: a scene has ceil(2 * boundary samples / 32)
// chunks; the sample counts are known on the device only, so every block
// forms the item list itself
template <class Q>
__global__ void __launch_bounds__(512, 1)
    k_edge_eval_batch(const BatchScene *B, int nb, const int *order, int spt, int *counter) {
  __shared__ int start[DVG_BATCH_MAX + 1];
  int lane = threadIdx.x & 31;
  Q *q = warp_queue_local<Q>();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int r = 0; r < nb; r++) {
      start[r] = run;
      const BatchScene &b = B[__ldg(&order[r])];
      int T = b.S.tiles_x * b.S.tiles_y * DVG_EDGE_CELLS;
      int chunks = (2 * __ldg(&b.E.tile_start[T]) + 31) / 32;
      run += (chunks + spt - 1) / spt;
    }
    start[nb] = run;
  }
  __syncthreads();
  int total = start[nb];
  #pragma unroll 1
  for (int item = batch_next(counter, lane); item < total; item = batch_next(counter, lane)) {
    int r = batch_range_of(start, nb, item);
    const BatchScene &b = B[__ldg(&order[r])];
    DevRender R = load_filter(b.R, nullptr);
    long long c0 = (long long)(item - start[r]) * spt;
    #pragma unroll 1
    for (int k = 0; k < spt; k++) edge_eval_one<true>(b.S, R, b.E, (c0 + k) * 32 + lane, q, lane);
  }
}

// the deferred segment tests of every scene of the batch: their quintics
// and root brackets (as k_edge_jobs), scene after scene
__global__ void __launch_bounds__(256) k_edge_jobs_batch(const BatchScene *B, int nb, const int *order) {
  for (int r = 0; r < nb; r++) {
    const BatchScene &b = B[__ldg(&order[r])];
    if (b.E.job_a) edge_jobs_all(b.S, b.E);
  }
}
// their root brackets' walks (as k_edge_roots), scene after scene
__global__ void __launch_bounds__(256) k_edge_roots_batch(const BatchScene *B, int nb, const int *order) {
  for (int r = 0; r < nb; r++) {
    const BatchScene &b = B[__ldg(&order[r])];
    if (b.E.job_a) edge_roots_all(b.S, b.E);
  }
}

static inline int tiles_of(const DevRender &R) {
  return ((R.w + DVG_TILE - 1) / DVG_TILE) * ((R.h + DVG_TILE - 1) / DVG_TILE);
}
static inline unsigned blocks_of(long long n) { return (unsigned)((n + 255) / 256); }
// grid of a sample pass run with blocks of `threads` (block_group)
static inline dim3 group_grid(const DevRender &R, int threads) {
  int k = threads / 256, tiles = tiles_of(R);
  return R.spp >= k ? dim3(tiles, (R.spp + k - 1) / k) : dim3((tiles + k - 1) / k, R.spp);
}

// Opts kernel `id` (one of QueueKernel) into kQueueBytes of dynamic shared
// memory, once per device (devices 0-63; the others every call).
enum QueueKernel {
  QK_FWD, QK_FWD_WIDE, QK_FWD_FILL, QK_BWD, QK_EDGE_PAIRS, QK_EDGE_PAIRS_WIDE, QK_EDGE, QK_FWD_BATCH, QK_FWD_BATCH_WIDE,
  QK_BWD_BATCH, QK_EDGE_BATCH, QK_EDGE_BATCH_WIDE, QK_COUNT
};
template <class K>
static void allow_queues(K *kernel, int id, int bytes = kQueueBytes) {
  static std::atomic<unsigned long long> done[QK_COUNT];
  int dev = 0;
  cudaGetDevice(&dev);
  unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done[id].load() & bit)) return;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  done[id].fetch_or(bit);
}

// SM count of the current device
static int sm_count() {
  static std::mutex mu;
  static int sms[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 0 || dev >= 64) dev = 0;
  if (sms[dev] <= 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sms[dev] = v > 0 ? v : 128;
  }
  return sms[dev];
}

static unsigned persistent_grid(int ctas_per_sm) {
  return (unsigned)(sm_count() * (ctas_per_sm > 0 ? ctas_per_sm : 1));
}

void launch_weight(const DevScene &S, const DevRender &R, cudaStream_t st) {
  k_weight<<<blocks_of((long long)R.w * R.h), 256, 0, st>>>(R, S);
}
void launch_sample_fwd(const DevScene &S, const DevRender &R, float4 *samples, cudaStream_t st,
                       const EdgeRecords *D) {
  if (R.hit_chunk_count) cudaMemsetAsync(R.hit_chunk_count, 0, sizeof(int), st);
  EdgeRecords none{};
  if (R.prefilter) {
    int threads = 256 * R.spp >= DVG_PF_FWD_THREADS ? DVG_PF_FWD_THREADS : 256;
    dim3 grid(tiles_of(R), (256 * R.spp + threads - 1) / threads);
    k_sample_fwd<true, WarpQueue><<<grid, threads, 0, st>>>(S, R, samples, none);
  } else {
    bool defer = D && D->job_a;
    if (defer) cudaMemsetAsync(D->counts, 0, 8 * sizeof(int), st);
    int threads = 256 * R.spp >= DVG_FWD_THREADS ? DVG_FWD_THREADS : 256;
    dim3 grid(tiles_of(R), (256 * R.spp + threads - 1) / threads);
    if (S.wide_queues) {
      constexpr int qb = queue_local_bytes<WarpQueueWide>();
      allow_queues(k_sample_fwd<false, WarpQueueWide>, QK_FWD_WIDE, DVG_FWD_THREADS / 32 * qb);
      k_sample_fwd<false, WarpQueueWide><<<grid, threads, threads / 32 * qb, st>>>(S, R, samples, defer ? *D : none);
    } else if (S.fill_heavy) {
      constexpr int qb = queue_local_bytes<WarpQueue>();
      auto *k = k_sample_fwd<false, WarpQueue, DVG_FWD_FILL_BLOCKS>;
      allow_queues(k, QK_FWD_FILL, DVG_FWD_THREADS / 32 * qb);
      k<<<grid, threads, threads / 32 * qb, st>>>(S, R, samples, defer ? *D : none);
    } else {
      constexpr int qb = queue_local_bytes<WarpQueue>();
      allow_queues(k_sample_fwd<false, WarpQueue>, QK_FWD, DVG_FWD_THREADS / 32 * qb);
      k_sample_fwd<false, WarpQueue><<<grid, threads, threads / 32 * qb, st>>>(S, R, samples, defer ? *D : none);
    }
    if (defer) {
      k_edge_jobs<<<persistent_grid(8), 256, 0, st>>>(S, *D);
      k_edge_roots<<<persistent_grid(6), 256, 0, st>>>(S, *D);
      k_fwd_finish<<<persistent_grid(8), 256, 0, st>>>(S, R, *D, samples);
    }
  }
}
void launch_hit_check(const float *params, const float *fwd_params, int n, unsigned *stale, cudaStream_t st) {
  int blocks = (n + 255) / 256;
  k_hit_check<<<blocks < 1 ? 1 : (blocks > 1216 ? 1216 : blocks), 256, 0, st>>>(params, fwd_params, n, stale);
}
void launch_resolve(const DevRender &R, const float4 *samples, float *image, cudaStream_t st) {
  k_resolve<<<blocks_of((long long)R.w * R.h), 256, 0, st>>>(R, samples, image);
}
void launch_sample_bwd(const DevScene &S, const DevRender &R, float4 *dbg_val, int *dbg_flag, cudaStream_t st) {
  cudaMemsetAsync(R.deep_count, 0, sizeof(int), st);
  if (R.prefilter) {
    k_sample_bwd<true><<<group_grid(R, DVG_PF_BWD_THREADS), DVG_PF_BWD_THREADS, 0, st>>>(S, R, dbg_val, dbg_flag);
    k_sample_bwd_deep_pf<<<sm_count() * 2, 256, 0, st>>>(S, R, dbg_val, dbg_flag);
  } else {
    allow_queues(k_sample_bwd<false>, QK_BWD, DVG_BWD_THREADS / 32 * (int)sizeof(WarpQueue));
    k_sample_bwd<false><<<group_grid(R, DVG_BWD_THREADS), DVG_BWD_THREADS, DVG_BWD_THREADS / 32 * sizeof(WarpQueue),
                          st>>>(S, R, dbg_val, dbg_flag);
    k_sample_bwd_deep<<<sm_count() * 4, 32, 0, st>>>(S, R, dbg_val, dbg_flag);
  }
}
void launch_bg_combine(const DevScene &S, const DevRender &R, const float4 *dbg_val, const int *dbg_flag,
                       cudaStream_t st) {
  k_bg_combine<<<blocks_of((long long)R.w * R.h), 256, 0, st>>>(S, R, dbg_val, dbg_flag);
}

void launch_edge_setup(const DevScene &S, const DevRender &R, const EdgeRecords &E, cudaStream_t st) {
  long long n = (long long)R.w * R.h * R.spp;
  cudaMemsetAsync(E.tile_count, 0, sizeof(int) * S.tiles_x * S.tiles_y * DVG_EDGE_CELLS, st);
  k_edge_sample<<<blocks_of(n), 256, 0, st>>>(S, R, E);
  k_edge_scan<<<1, 1024, 0, st>>>(S, E);
  k_edge_order<<<blocks_of(n), 256, 0, st>>>(E, (int)n);
  if (S.num_groups >= 8 && E.job_a) cudaMemsetAsync(E.counts, 0, 8 * sizeof(int), st);
}
void launch_edge_eval(const DevScene &S, const DevRender &R, const EdgeRecords &E, cudaStream_t st) {
  long long n = (long long)R.w * R.h * R.spp;
  if (S.num_groups >= 8) {  // two lanes per sample
    unsigned blocks = (unsigned)((2 * n + DVG_EDGE_THREADS - 1) / DVG_EDGE_THREADS);
    if (S.wide_queues) {
      constexpr int qb = queue_local_bytes<WarpQueueWide>();
      allow_queues(k_edge_eval<true, WarpQueueWide>, QK_EDGE_PAIRS_WIDE, DVG_EDGE_THREADS / 32 * qb);
      k_edge_eval<true, WarpQueueWide><<<blocks, DVG_EDGE_THREADS, DVG_EDGE_THREADS / 32 * qb, st>>>(S, R, E);
    } else {
      constexpr int qb = queue_local_bytes<WarpQueue>();
      allow_queues(k_edge_eval<true, WarpQueue>, QK_EDGE_PAIRS, DVG_EDGE_THREADS / 32 * qb);
      k_edge_eval<true, WarpQueue><<<blocks, DVG_EDGE_THREADS, DVG_EDGE_THREADS / 32 * qb, st>>>(S, R, E);
    }
    if (E.job_a) {
      k_edge_jobs<<<persistent_grid(8), 256, 0, st>>>(S, E);
      k_edge_roots<<<persistent_grid(6), 256, 0, st>>>(S, E);
      k_edge_finish<<<persistent_grid(8), 256, 0, st>>>(S, R, E);
    }
  } else {
    constexpr int qb = queue_local_bytes<WarpQueue>();
    allow_queues(k_edge_eval<false, WarpQueue>, QK_EDGE, DVG_EDGE1_THREADS / 32 * qb);
    k_edge_eval<false, WarpQueue><<<(unsigned)((n + DVG_EDGE1_THREADS - 1) / DVG_EDGE1_THREADS), DVG_EDGE1_THREADS,
                                    DVG_EDGE1_THREADS / 32 * qb, st>>>(S, R, E);
  }
}
void launch_edge(const DevScene &S, const DevRender &R, const EdgeRecords &E, cudaStream_t st) {
  launch_edge_setup(S, R, E, st);
  launch_edge_eval(S, R, E, st);
}

// The batched walks run ctas_per_sm blocks of 512 / ctas_per_sm threads per
// SM (128 registers a thread either way), with the wide queues when every
// scene of the batch is stroke-heavy.
void launch_batch_sample_fwd(const BatchScene *B, int nb, const int *order, const int *item_start, int spt,
                             int ctas_per_sm, int *counter, bool wide, cudaStream_t st) {
  cudaMemsetAsync(counter, 0, sizeof(int), st);
  int threads = ctas_per_sm >= 2 ? 256 : 512;
  if (wide) {
    constexpr int qb = queue_local_bytes<WarpQueueWide>();
    allow_queues(k_sample_fwd_batch<WarpQueueWide>, QK_FWD_BATCH_WIDE, 512 / 32 * qb);
    k_sample_fwd_batch<WarpQueueWide><<<persistent_grid(ctas_per_sm), threads, threads / 32 * qb, st>>>(
        B, nb, order, item_start, spt, counter);
  } else {
    constexpr int qb = queue_local_bytes<WarpQueue>();
    allow_queues(k_sample_fwd_batch<WarpQueue>, QK_FWD_BATCH, 512 / 32 * qb);
    k_sample_fwd_batch<WarpQueue><<<persistent_grid(ctas_per_sm), threads, threads / 32 * qb, st>>>(
        B, nb, order, item_start, spt, counter);
  }
}
void launch_batch_sample_bwd(const BatchScene *B, int nb, const int *order, const int *item_start, int spt,
                             int ctas_per_sm, int *counter, cudaStream_t st) {
  cudaMemsetAsync(counter, 0, sizeof(int), st);
  allow_queues(k_sample_bwd_batch, QK_BWD_BATCH);
  k_sample_bwd_batch<<<persistent_grid(ctas_per_sm), 256, kQueueBytes, st>>>(B, nb, order, item_start, spt, counter);
  k_sample_bwd_deep_batch<<<persistent_grid(4), 32, 0, st>>>(B, nb, order);
}
void launch_batch_edge(const BatchScene *B, int nb, const int *order, int spt, int ctas_per_sm, int *counter,
                       bool wide, cudaStream_t st) {
  cudaMemsetAsync(counter, 0, sizeof(int), st);
  int threads = ctas_per_sm >= 2 ? 256 : 512;
  if (wide) {
    constexpr int qb = queue_local_bytes<WarpQueueWide>();
    allow_queues(k_edge_eval_batch<WarpQueueWide>, QK_EDGE_BATCH_WIDE, 512 / 32 * qb);
    k_edge_eval_batch<WarpQueueWide><<<persistent_grid(ctas_per_sm), threads, threads / 32 * qb, st>>>(
        B, nb, order, spt, counter);
  } else {
    constexpr int qb = queue_local_bytes<WarpQueue>();
    allow_queues(k_edge_eval_batch<WarpQueue>, QK_EDGE_BATCH, 512 / 32 * qb);
    k_edge_eval_batch<WarpQueue><<<persistent_grid(ctas_per_sm), threads, threads / 32 * qb, st>>>(
        B, nb, order, spt, counter);
  }
  k_edge_jobs_batch<<<persistent_grid(8), 256, 0, st>>>(B, nb, order);
  k_edge_roots_batch<<<persistent_grid(6), 256, 0, st>>>(B, nb, order);
  k_edge_finish_batch<<<persistent_grid(8), 256, 0, st>>>(B, nb, order);
}
void launch_sdf(const DevScene &S, const DevRender &R, const float *eval_positions, int num_eval, float *sdf,
                const float *d_sdf, cudaStream_t st) {
  long long n = eval_positions ? num_eval : (long long)R.w * R.h * R.spp;
  if (n <= 0) return;
  k_sdf<<<blocks_of(n), 256, 0, st>>>(S, R, eval_positions, num_eval, sdf, d_sdf);
}

}  // namespace dvg
