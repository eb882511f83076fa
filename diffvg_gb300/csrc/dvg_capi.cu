// C ABI of libdiffvg_gb300 (include/diffvg_gb300.h): scene handles that keep
// the topology and all scratch arenas resident on the device, and the
// forward / backward entry points that replace diffvg.Scene + diffvg.render
// (diffvg.cpp:1477-1649, 1777-1789; scene.cpp:919-1035).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "dvg_internal.h"

namespace dvg {

// last error of this thread; a fixed buffer, so that reporting an error
// allocates nothing
thread_local char g_last_error[512];

int fail(int status, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(DVG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void clear_error() { g_last_error[0] = 0; }

}  // namespace dvg

namespace {

using dvg::cuda_fail;
using dvg::fail;

// grow-only device buffer
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t nb = need + need / 4 + 256;
    cudaError_t e = cudaMalloc(&ptr, nb);
    if (e == cudaSuccess) bytes = nb;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
};

}  // namespace

struct DvgScene {
  int device = 0;
  DvgSceneDesc d{};
  int tiles_x = 1, tiles_y = 1;
  int num_total = 0;
  DevBuf topo, derived, tiles;
  int tile_cap = 0;
  // carved from `topo`
  int *shape_info = nullptr, *segment_ctrl = nullptr, *seg_point = nullptr, *group_info = nullptr;
  int *group_shapes = nullptr, *smp_shape = nullptr, *smp_group = nullptr;
  // carved from `derived`
  float *c2s = nullptr, *g_max_radius = nullptr, *s_length = nullptr;
  float4 *g_local_box = nullptr, *g_canvas_box = nullptr, *s_box = nullptr, *seg_box = nullptr;
  float *seg_r = nullptr, *seg_pmf = nullptr, *seg_cdf = nullptr, *smp_cdf = nullptr, *smp_pmf = nullptr;
  int *seg_order = nullptr, *tile_start = nullptr, *tile_count = nullptr, *scratch = nullptr;
  int4 *g_tile_range = nullptr;
  int num_records = 0;  // stroke records (k_rec_fill)
  int num_paths = 0;    // path shapes
  int2 *g_rec = nullptr;
  float4 *rec_box = nullptr;
  int4 *rec_a = nullptr, *rec_b = nullptr;
  float *rec_r = nullptr;
  float4 *rec_cbox = nullptr;
  float2 *seg_tpts = nullptr;
  float *seg_th = nullptr;
  // y-band segment lists of long paths (all null when no path has them)
  int4 *shape_band = nullptr;  // topology
  float2 *band_geo = nullptr;
  int *band_n = nullptr, *band_start = nullptr, *band_seg = nullptr;
  unsigned *err = nullptr;  // [0] status bits, [1] tile-list length
  // image-sized arenas
  DevBuf weight, samples, dbg_val, dbg_flag, edge;
  // backward: the count and list of the samples left to the deep pass
  DevBuf deep;
  // the scene's own parameter arena (dvg_scene_update_params), read by calls
  // whose DvgRenderArgs.params is NULL
  DevBuf own_params;
  bool has_params = false;
  bool wide_queues = false;  // three quarters or more of the groups stroked (DevScene::wide_queues)
  bool fill_heavy = false;   // 64 or more groups, a quarter or less stroked (DevScene::fill_heavy)
  // fragment cache of the last image forward (no prefiltering): per-sample
  // hit keys and counts, a copy of its parameters and the stale flag the
  // backward sets when its parameters differ
  DevBuf hits;
  bool hit_live = false, hit_pf = false;
  size_t hit_chunks_seen = 0;  // chunks the last synchronous forward asked for
  bool hit_pf_seen = false;    // ... with prefiltering
  int hit_w = 0, hit_h = 0, hit_nsx = 0, hit_nsy = 0;
  uint64_t hit_seed = 0;
  unsigned *h_status = nullptr;  // pinned mirror of err[0..1]
  bool prepared = false;
  // per-kernel timing (dvg_scene_profile)
  bool profiling = false;
  struct Pending { int kid; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  double total_ms[16] = {0};
  long long launches[16] = {0};
};

namespace {

template <typename T>
T *carve(char *&p, size_t n) {
  uintptr_t a = (reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255);
  T *r = reinterpret_cast<T *>(a);
  p = reinterpret_cast<char *>(a + sizeof(T) * (n > 0 ? n : 1));
  return r;
}

size_t carve_size(const std::vector<size_t> &bytes) {
  size_t s = 0;
  for (size_t b : bytes) s += ((b > 0 ? b : 4) + 255) / 256 * 256 + 256;
  return s + 256;
}

enum { K_PREPARE, K_WEIGHT, K_SAMPLE_FWD, K_RESOLVE, K_SAMPLE_BWD, K_BG_COMBINE, K_EDGE, K_SDF, K_COUNT };
const char *const kKernelNames[K_COUNT] = {"prepare", "weight", "sample_fwd", "resolve",
                                           "sample_bwd", "bg_combine", "edge", "sdf"};

cudaEvent_t take_event(DvgScene *sc) {
  if (!sc->event_pool.empty()) {
    cudaEvent_t e = sc->event_pool.back();
    sc->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Runs `launch` (kernel launches on st); with profiling on, brackets it with
// two events on the same stream.
template <class F>
void timed(DvgScene *sc, int kid, cudaStream_t st, F launch) {
  if (!sc->profiling) { launch(); return; }
  cudaEvent_t a = take_event(sc), b = take_event(sc);
  if (a) cudaEventRecord(a, st);
  launch();
  if (b) cudaEventRecord(b, st);
  if (a && b) sc->pending.push_back({kid, a, b});
}

}  // namespace

namespace dvg {

// Host-side checks of a scene description; writes the first point of every
// path segment to seg_point when it is not NULL.  Allocates nothing.
int validate_desc(const DvgSceneDesc *d, int *seg_point) {
  if (!d) return fail(DVG_ERR_INVALID, "scene description is NULL");
  if (d->canvas_width <= 0 || d->canvas_height <= 0) return fail(DVG_ERR_INVALID, "canvas size must be positive");
  if (d->num_shapes < 0 || d->num_groups < 0 || d->num_params < 1 || d->total_segments < 0 ||
      d->total_group_shapes < 0)
    return fail(DVG_ERR_INVALID, "negative counts in scene description");
  if ((d->num_shapes > 0 && !d->shape_info) || (d->num_groups > 0 && !d->group_info) ||
      (d->total_segments > 0 && !d->segment_ctrl) || (d->total_group_shapes > 0 && !d->group_shapes))
    return fail(DVG_ERR_INVALID, "missing topology array");
  if (d->filter_type < DVG_BOX || d->filter_type > DVG_GAUSSIAN) return fail(DVG_ERR_INVALID, "unknown filter type");
  auto in_params = [&](long long off, long long n) { return off >= 0 && n >= 0 && off + n <= d->num_params; };
  if (!in_params(d->filter_radius_off, 1)) return fail(DVG_ERR_INVALID, "filter radius offset out of range");
  for (int s = 0; s < d->num_shapes; s++) {
    const int32_t *si = d->shape_info + (size_t)s * DVG_SHAPE_INFO_STRIDE;
    int kind = si[DVG_SHAPE_KIND], po = si[DVG_SHAPE_PARAM_OFF];
    if (!in_params(si[DVG_SHAPE_STROKE_WIDTH_OFF], 1))
      return fail(DVG_ERR_INVALID, "shape %d: stroke width offset out of range", s);
    if (kind == DVG_CIRCLE) {
      if (!in_params(po, 3)) return fail(DVG_ERR_INVALID, "circle parameters out of range");
    } else if (kind == DVG_ELLIPSE || kind == DVG_RECT) {
      if (!in_params(po, 4)) return fail(DVG_ERR_INVALID, "shape parameters out of range");
    } else if (kind == DVG_PATH) {
      int np = si[DVG_SHAPE_NUM_POINTS], nseg = si[DVG_SHAPE_NUM_SEGMENTS], so = si[DVG_SHAPE_SEG_OFF];
      int th = si[DVG_SHAPE_THICKNESS_OFF];
      if (np < 0 || nseg < 0 || so < 0 || (long long)so + nseg > d->total_segments)
        return fail(DVG_ERR_INVALID, "path %d: segment range out of bounds", s);
      if (!in_params(po, 2LL * np)) return fail(DVG_ERR_INVALID, "path points out of range");
      if (th >= 0 && !in_params(th, np)) return fail(DVG_ERR_INVALID, "path thickness out of range");
      if (nseg > 0 && np < 1) return fail(DVG_ERR_INVALID, "path with segments but no points");
      int pid = 0;
      for (int i = 0; i < nseg; i++) {
        int nc = d->segment_ctrl[so + i];
        if (nc < 0 || nc > 2) return fail(DVG_ERR_INVALID, "num_control_points entries must be 0, 1 or 2");
        if (pid + nc >= np) return fail(DVG_ERR_INVALID, "num_control_points does not fit the number of points");
        if (seg_point) seg_point[(size_t)so + i] = pid;
        pid += nc + 1;
      }
    } else {
      return fail(DVG_ERR_INVALID, "unknown shape kind %d", kind);
    }
  }
  for (int g = 0; g < d->num_groups; g++) {
    const int32_t *gi = d->group_info + (size_t)g * DVG_GROUP_INFO_STRIDE;
    int nsh = gi[DVG_GROUP_NUM_SHAPES], off = gi[DVG_GROUP_SHAPES_OFF];
    if (nsh < 1 || off < 0 || (long long)off + nsh > d->total_group_shapes)
      return fail(DVG_ERR_INVALID, "group %d: shape list out of range", g);
    for (int k = 0; k < nsh; k++) {
      int s = d->group_shapes[off + k];
      if (s < 0 || s >= d->num_shapes) return fail(DVG_ERR_INVALID, "group refers to a shape id out of range");
    }
    for (int which = 0; which < 2; which++) {
      int kind = gi[which ? DVG_GROUP_STROKE_KIND : DVG_GROUP_FILL_KIND];
      int po = gi[which ? DVG_GROUP_STROKE_OFF : DVG_GROUP_FILL_OFF];
      int k = gi[which ? DVG_GROUP_STROKE_STOPS : DVG_GROUP_FILL_STOPS];
      if (kind == DVG_PAINT_NONE) continue;
      if (kind == DVG_CONSTANT) {
        if (!in_params(po, 4)) return fail(DVG_ERR_INVALID, "constant paint out of range");
      } else if (kind == DVG_LINEAR || kind == DVG_RADIAL) {
        if (k < 1 || !in_params(po, 4 + 5LL * k)) return fail(DVG_ERR_INVALID, "gradient paint out of range");
      } else {
        return fail(DVG_ERR_INVALID, "unknown paint kind");
      }
    }
    if (!in_params(gi[DVG_GROUP_XFORM_OFF], 9)) return fail(DVG_ERR_INVALID, "group transform out of range");
  }
  return DVG_OK;
}

// Number of stroke records of a (validated) description: per stroke group
// and shape, one per path segment, or one for a shape that is not tested
// segment by segment (k_rec_fill).  Allocates nothing.
int count_stroke_records(const DvgSceneDesc *d) {
  long long n = 0;
  for (int g = 0; g < d->num_groups; g++) {
    const int32_t *gi = d->group_info + (size_t)g * DVG_GROUP_INFO_STRIDE;
    if (gi[DVG_GROUP_STROKE_KIND] == DVG_PAINT_NONE) continue;
    for (int k = 0; k < gi[DVG_GROUP_NUM_SHAPES]; k++) {
      const int32_t *si = d->shape_info + (size_t)d->group_shapes[gi[DVG_GROUP_SHAPES_OFF] + k] * DVG_SHAPE_INFO_STRIDE;
      bool per_segment = si[DVG_SHAPE_KIND] == DVG_PATH && !(si[DVG_SHAPE_FLAGS] & 2);
      n += per_segment ? si[DVG_SHAPE_NUM_SEGMENTS] : 1;
    }
  }
  return (int)n;
}

}  // namespace dvg

namespace {

using dvg::validate_desc;

DevScene make_dev(DvgScene *sc, const float *params) {
  DevScene S;
  S.W = sc->d.canvas_width;
  S.H = sc->d.canvas_height;
  S.num_shapes = sc->d.num_shapes;
  S.num_groups = sc->d.num_groups;
  S.num_segments = sc->d.total_segments;
  S.num_total = sc->num_total;
  S.shape_info = sc->shape_info;
  S.segment_ctrl = sc->segment_ctrl;
  S.seg_point = sc->seg_point;
  S.group_info = sc->group_info;
  S.group_shapes = sc->group_shapes;
  S.smp_shape = sc->smp_shape;
  S.smp_group = sc->smp_group;
  S.P = params;
  S.c2s = sc->c2s;
  S.g_local_box = sc->g_local_box;
  S.g_canvas_box = sc->g_canvas_box;
  S.g_max_radius = sc->g_max_radius;
  S.s_box = sc->s_box;
  S.s_length = sc->s_length;
  S.seg_box = sc->seg_box;
  S.seg_r = sc->seg_r;
  S.g_rec = sc->g_rec;
  S.rec_box = sc->rec_box;
  S.rec_a = sc->rec_a;
  S.rec_b = sc->rec_b;
  S.rec_r = sc->rec_r;
  S.rec_cbox = sc->rec_cbox;
  S.seg_tpts = sc->seg_tpts;
  S.seg_th = sc->seg_th;
  S.wide_queues = sc->wide_queues ? 1 : 0;
  S.fill_heavy = sc->fill_heavy ? 1 : 0;
  S.num_paths = sc->num_paths;
  S.num_records = sc->num_records;
  S.shape_band = sc->shape_band;
  S.band_geo = sc->band_geo;
  S.band_n = sc->band_n;
  S.band_start = sc->band_start;
  S.band_seg = sc->band_seg;
  S.seg_pmf = sc->seg_pmf;
  S.seg_cdf = sc->seg_cdf;
  S.seg_order = sc->seg_order;
  S.smp_cdf = sc->smp_cdf;
  S.smp_pmf = sc->smp_pmf;
  S.tiles_x = sc->tiles_x;
  S.tiles_y = sc->tiles_y;
  S.tile_start = sc->tile_start;
  S.tile_list = reinterpret_cast<int *>(sc->tiles.ptr);
  S.tile_mask = reinterpret_cast<unsigned *>(sc->tiles.ptr) + sc->tile_cap;
  S.scratch = sc->scratch;
  S.err = sc->err;
  return S;
}

// a's parameters: a->params, or the scene's own arena when that is NULL
const DvgRenderArgs *with_params(DvgScene *sc, const DvgRenderArgs *a, DvgRenderArgs &tmp) {
  if (!sc || !a || a->params || !sc->has_params) return a;
  tmp = *a;
  tmp.params = reinterpret_cast<const float *>(sc->own_params.ptr);
  return &tmp;
}

int check_args(DvgScene *sc, const DvgRenderArgs *a) {
  if (!sc) return fail(DVG_ERR_INVALID, "scene is NULL");
  if (!a) return fail(DVG_ERR_INVALID, "render arguments are NULL");
  if (a->width <= 0 || a->height <= 0 || a->num_samples_x <= 0 || a->num_samples_y <= 0)
    return fail(DVG_ERR_INVALID, "image size and sample counts must be positive");
  if ((long long)a->width * a->height * a->num_samples_x * a->num_samples_y > 0x7fffffffLL)
    return fail(DVG_ERR_INVALID, "more than 2^31-1 samples per call (the reference indexes samples with int)");
  if (!a->params) return fail(DVG_ERR_INVALID, "params is NULL and the scene has no arena of its own");
  if (a->background && (reinterpret_cast<uintptr_t>(a->background) & 15u))
    return fail(DVG_ERR_INVALID, "background must be 16-byte aligned");
  return DVG_OK;
}

DevRender make_render(DvgScene *sc, const DvgRenderArgs *a) {
  DevRender R;
  R.w = a->width;
  R.h = a->height;
  R.nsx = a->num_samples_x;
  R.nsy = a->num_samples_y;
  R.spp = R.nsx * R.nsy;
  R.seed = a->seed;
  R.prefilter = a->use_prefiltering ? 1 : 0;
  R.ftype = sc->d.filter_type;
  R.fr_ptr = a->params + sc->d.filter_radius_off;
  R.fr = 0.f;  // read on the device (load_filter)
  R.ri = 0;
  R.background = a->background;
  R.weight = reinterpret_cast<float *>(sc->weight.ptr);
  R.d_image = nullptr;
  R.d_params = nullptr;
  R.d_background = nullptr;
  R.d_translation = nullptr;
  R.filter_radius_off = sc->d.filter_radius_off;
  return R;
}

// scoped device switch
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

int prepare(DvgScene *sc, const DevScene &S, const DvgRenderArgs *a, cudaStream_t st) {
  cudaError_t e;
  if (!(a->flags & DVG_FLAG_NO_SYNC)) {
    // a synchronous call reports only its own failures; with NO_SYNC the
    // bits stay latched until dvg_scene_sync()
    e = cudaMemsetAsync(sc->err, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return cuda_fail(e, "clearing the status word");
  }
  if ((a->flags & DVG_FLAG_REUSE_PREP) && sc->prepared) return DVG_OK;
  timed(sc, K_PREPARE, st, [&] {
    e = dvg::launch_prepare(S, sc->tile_cap, reinterpret_cast<int *>(sc->err + 1), sc->g_tile_range, sc->tile_count,
                            st);
  });
  if (e != cudaSuccess) return cuda_fail(e, "scene preparation launch");
  sc->prepared = true;
  return DVG_OK;
}

struct HitArena {
  int *keys;  // [DVG_HIT_SLOTS][n] keys, or with prefiltering [DVG_PF_SLOTS][n] fragments
  unsigned short *cnt;
  float *params;
  unsigned *stale;
  int *chunks;       // keys and next chunk, or with prefiltering the next chunk only
  void *pf_chunks;   // prefiltering: [chunk_cap][DVG_PF_CHUNK] fragments
  int *first, *chunk_count;
  int chunk_cap;
};

// per sample: DVG_HIT_SLOTS fragment keys, or with prefiltering DVG_PF_SLOTS whole fragments
size_t hit_slot_bytes(bool prefilter) { return prefilter ? DVG_PF_SLOTS * DVG_PF_BYTES : DVG_HIT_SLOTS * sizeof(int); }

// Chunks for the entries past the slots: without prefiltering one per two
// samples (8 more keys per sample on average), with prefiltering one per
// sixteen samples, or what the last synchronous forward asked for with a
// quarter to spare, up to what a sample of the reference's maximum
// fragment count needs.  Samples that find none left are recomputed by the
// backward pass.
size_t hit_chunk_cap(DvgScene *sc, size_t n, bool prefilter) {
  size_t base = prefilter ? n / 16 + 64 : n / 2 + 64;
  size_t most = prefilter ? (size_t)(DVG_MAX_PREFILTER_FRAGMENTS - DVG_PF_SLOTS) / DVG_PF_CHUNK * n + 64
                          : (size_t)(DVG_MAX_FRAGMENTS - DVG_HIT_SLOTS) / DVG_HIT_CHUNK * n + 64;
  size_t seen = sc->hit_pf_seen == prefilter ? sc->hit_chunks_seen : 0;
  return std::min(std::max(base, seen + seen / 4), most);
}

size_t hit_bytes(DvgScene *sc, size_t n, bool prefilter) {
  size_t cap = hit_chunk_cap(sc, n, prefilter);
  return carve_size({hit_slot_bytes(prefilter) * n, n * sizeof(unsigned short), (size_t)sc->d.num_params * sizeof(float),
                     sizeof(unsigned), cap * (prefilter ? sizeof(int) : (DVG_HIT_CHUNK + 1) * sizeof(int)),
                     prefilter ? cap * DVG_PF_CHUNK * DVG_PF_BYTES : 0, n * sizeof(int), sizeof(int)});
}

HitArena hit_arena(DvgScene *sc, size_t n, bool prefilter) {
  char *p = reinterpret_cast<char *>(sc->hits.ptr);
  size_t cap = hit_chunk_cap(sc, n, prefilter);
  HitArena h;
  h.keys = carve<int>(p, hit_slot_bytes(prefilter) * n / sizeof(int));
  h.cnt = carve<unsigned short>(p, n);
  h.params = carve<float>(p, sc->d.num_params);
  h.stale = carve<unsigned>(p, 1);
  h.chunks = carve<int>(p, cap * (prefilter ? 1 : DVG_HIT_CHUNK + 1));
  h.pf_chunks = carve<char>(p, prefilter ? cap * DVG_PF_CHUNK * DVG_PF_BYTES : 0);
  if (!prefilter) h.pf_chunks = nullptr;
  h.first = carve<int>(p, n);
  h.chunk_count = carve<int>(p, 1);
  h.chunk_cap = (int)cap;
  return h;
}

// R's view of the cache
void set_hit_cache(DevRender &R, const HitArena &h, bool prefilter) {
  if (prefilter) {
    R.pf_frags = h.keys;
    R.pf_chunk_frags = h.pf_chunks;
  } else {
    R.hit_keys = h.keys;
  }
  R.hit_cnt = h.cnt;
  R.hit_chunks = h.chunks;
  R.hit_first = h.first;
  R.hit_chunk_count = h.chunk_count;
  R.hit_chunk_cap = h.chunk_cap;
}

// After a synchronous forward: when its samples asked for more chunks than
// the cache holds, the cache is enlarged now (between calls, never while a
// graph may be capturing one) and the keys just written are dropped.
void grow_hit_chunks(DvgScene *sc, size_t n, bool pf) {
  HitArena h = hit_arena(sc, n, pf);
  int asked = 0;
  if (cudaMemcpy(&asked, h.chunk_count, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return;
  if (asked <= h.chunk_cap) return;
  sc->hit_chunks_seen = (size_t)asked;
  sc->hit_pf_seen = pf;
  sc->hit_live = false;
  if (sc->hits.ensure(hit_bytes(sc, n, pf)) != cudaSuccess) {
    cudaGetLastError();
    sc->hit_chunks_seen = 0;  // keep the smaller cache
    sc->hits.ensure(hit_bytes(sc, n, pf));
  }
}

bool hit_matches(const DvgScene *sc, const DvgRenderArgs *a) {
  return sc->hit_live && sc->hit_pf == (a->use_prefiltering != 0) && sc->hit_w == a->width &&
         sc->hit_h == a->height && sc->hit_nsx == a->num_samples_x && sc->hit_nsy == a->num_samples_y &&
         sc->hit_seed == a->seed;
}

// Deferred fp64 walks of the paired boundary pass (scenes of 8+ groups):
// room for one job and four candidate fragments per boundary sample; a warp
// that finds no room solves its jobs in place.
bool edge_defers(const DvgScene *sc, size_t n) { return sc->d.num_groups >= 8 && n < (1u << 30); }
size_t edge_job_cap(size_t n) { return n; }
size_t edge_task_cap(size_t n) { return 2 * n; }
size_t edge_frag_cap(size_t n) { return 4 * n; }

size_t edge_bytes(DvgScene *sc, size_t n) {
  size_t T = (size_t)sc->tiles_x * sc->tiles_y * DVG_EDGE_CELLS;
  std::vector<size_t> b = {n * sizeof(float4), n * sizeof(float4), n * sizeof(int4), n * sizeof(float2),
                           n * sizeof(int), n * sizeof(int), n * sizeof(int), T * sizeof(int), (T + 1) * sizeof(int)};
  if (edge_defers(sc, n)) {
    size_t jc = edge_job_cap(n), fc = edge_frag_cap(n), tc = edge_task_cap(n);
    for (size_t x : {jc * sizeof(int4), jc * sizeof(float4), 2 * n * sizeof(int4), 2 * n * sizeof(unsigned),
                     2 * n * sizeof(float4), fc * sizeof(int2), n * sizeof(int), 5 * jc * sizeof(double),
                     tc * sizeof(int4), 8 * sizeof(int)})
      b.push_back(x);
  }
  return carve_size(b);
}

EdgeRecords edge_records(DvgScene *sc, size_t n) {
  size_t T = (size_t)sc->tiles_x * sc->tiles_y * DVG_EDGE_CELLS;
  char *p = reinterpret_cast<char *>(sc->edge.ptr);
  EdgeRecords E;
  E.a = carve<float4>(p, n);
  E.b = carve<float4>(p, n);
  E.c = carve<int4>(p, n);
  E.d = carve<float2>(p, n);
  E.key = carve<int>(p, n);
  E.rank = carve<int>(p, n);
  E.order = carve<int>(p, n);
  E.tile_count = carve<int>(p, T);
  E.tile_start = carve<int>(p, T + 1);
  if (edge_defers(sc, n)) {
    size_t jc = edge_job_cap(n), fc = edge_frag_cap(n), tc = edge_task_cap(n);
    E.job_a = carve<int4>(p, jc);
    E.job_b = carve<float4>(p, jc);
    E.dq = carve<int4>(p, 2 * n);
    E.dq_res = carve<unsigned>(p, 2 * n);
    E.dq_col = carve<float4>(p, 2 * n);
    E.frag = carve<int2>(p, fc);
    E.ds = carve<int>(p, n);
    E.job_q = carve<double>(p, 5 * jc);
    E.task = carve<int4>(p, tc);
    E.counts = carve<int>(p, 8);
    E.job_cap = (int)std::min(jc, (size_t)0x7fffffff);
    E.frag_cap = (int)std::min(fc, (size_t)0x7fffffff);
    E.task_cap = (int)std::min(tc, (size_t)0x7fffffff);
  }
  return E;
}

// Waits for the stream and maps the device status word to a DvgStatus.
// Returns 1 when the tile lists overflowed and were grown (the caller
// repeats the call).
int finish(DvgScene *sc, cudaStream_t st, bool *retry) {
  *retry = false;
  cudaError_t e = cudaMemcpyAsync(sc->h_status, sc->err, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "render");
  unsigned bits = sc->h_status[0];
  if (bits & DVG_EFLAG_SCENE_ZERO)
    return fail(DVG_ERR_SCENE, "The total length of the shape boundaries in the scene is equal or less than 0.");
  if (bits & DVG_EFLAG_SCENE_NAN)
    return fail(DVG_ERR_SCENE, "The total length of the shape boundaries in the scene is not a number.");
  if (bits & DVG_EFLAG_BIN_OVERFLOW) {
    size_t need = (size_t)sc->h_status[1];
    size_t cap = need + need / 2 + 1024;
    if (cap > 0x7fffffffu) return fail(DVG_ERR_CAPACITY, "tile candidate lists exceed 2^31 entries");
    e = sc->tiles.ensure(cap * 2 * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "growing the tile lists");
    sc->tile_cap = (int)(sc->tiles.bytes / (2 * sizeof(int)));
    sc->prepared = false;
    *retry = true;
    return DVG_OK;
  }
  if (bits & DVG_EFLAG_FILTER) return fail(DVG_ERR_INVALID, "filter radius must be in [0, 64]");
  if (bits & DVG_EFLAG_CAPACITY)
    return fail(DVG_ERR_CAPACITY,
                "a sample has more fragments than the reference's per-sample limit (256, or 64 with prefiltering)");
  if (bits & DVG_EFLAG_UNSUPPORTED)
    return fail(DVG_ERR_UNSUPPORTED,
                "unsupported input (the reference asserts on it): ellipse stroke/prefilter, prefiltered circle "
                "stroke, or a rotated rect edge");
  return DVG_OK;
}

}  // namespace

extern "C" {

const char *dvg_last_error(void) { return dvg::g_last_error; }

const char *dvg_version(void) { return "diffvg_gb300 0.1 (sm_103a)"; }

int dvg_scene_create(const DvgSceneDesc *desc, DvgScene **out_scene) {
  dvg::clear_error();
  if (!out_scene) return fail(DVG_ERR_INVALID, "out_scene is NULL");
  *out_scene = nullptr;
  std::vector<int> seg_point((size_t)(desc && desc->total_segments > 0 ? desc->total_segments : 1), 0);
  int st = validate_desc(desc, seg_point.data());
  if (st != DVG_OK) return st;
  DvgScene *sc = new DvgScene();
  sc->d = *desc;
  sc->d.shape_info = nullptr;
  sc->d.segment_ctrl = nullptr;
  sc->d.group_info = nullptr;
  sc->d.group_shapes = nullptr;
  cudaGetDevice(&sc->device);
  int S = desc->num_shapes, G = desc->num_groups, NSEG = desc->total_segments, NGS = desc->total_group_shapes;
  sc->tiles_x = (desc->canvas_width + DVG_TILE - 1) / DVG_TILE;
  sc->tiles_y = (desc->canvas_height + DVG_TILE - 1) / DVG_TILE;
  int T = sc->tiles_x * sc->tiles_y;
  // stroke-heavy scenes give the walks the wider segment-test queue; scenes of
  // many fills run the sampled forward at two blocks per SM (a single fill's
  // forward is short and measured slower with it: 27.5 -> 34 us)
  int stroked = 0;
  for (int g = 0; g < G; g++)
    stroked += desc->group_info[(size_t)g * DVG_GROUP_INFO_STRIDE + DVG_GROUP_STROKE_KIND] != DVG_PAINT_NONE ? 1 : 0;
  sc->wide_queues = G > 0 && 4 * (long long)stroked >= 3 * (long long)G;
  sc->fill_heavy = G >= 64 && 4 * (long long)stroked <= (long long)G;
  // (group, shape) pairs of the boundary CDF, in group order (scene.cpp:207-246)
  std::vector<int> smp_shape, smp_group;
  for (int g = 0; g < G; g++) {
    const int32_t *gi = desc->group_info + (size_t)g * DVG_GROUP_INFO_STRIDE;
    for (int k = 0; k < gi[DVG_GROUP_NUM_SHAPES]; k++) {
      smp_shape.push_back(desc->group_shapes[gi[DVG_GROUP_SHAPES_OFF] + k]);
      smp_group.push_back(g);
    }
  }
  sc->num_total = (int)smp_shape.size();
  int NT = sc->num_total;
  sc->num_records = dvg::count_stroke_records(desc);
  int NR = sc->num_records;
  for (int i = 0; i < S; i++)
    sc->num_paths += desc->shape_info[(size_t)i * DVG_SHAPE_INFO_STRIDE + DVG_SHAPE_KIND] == DVG_PATH ? 1 : 0;
  // band lists of the paths with DVG_BAND_MIN_SEGMENTS or more segments: up
  // to one band per four segments (4 to 128), room for each segment to meet
  // four bands on average
  std::vector<int4> shape_band(S > 0 ? S : 1, make_int4(0, 0, 0, 0));
  long long band_starts = 0, band_entries = 0;
  for (int i = 0; i < S; i++) {
    const int32_t *si = desc->shape_info + (size_t)i * DVG_SHAPE_INFO_STRIDE;
    int nseg = si[DVG_SHAPE_NUM_SEGMENTS];
    if (si[DVG_SHAPE_KIND] != DVG_PATH || nseg < DVG_BAND_MIN_SEGMENTS) continue;
    int nb = std::min(std::max(nseg / 4, 4), 128);
    int cap = 4 * nseg + 2 * nb;
    shape_band[i] = make_int4(nb, (int)band_starts, (int)band_entries, cap);
    band_starts += nb + 1;
    band_entries += cap;
  }
  if (band_starts + band_entries > 0x7fffffffLL) { delete sc; return fail(DVG_ERR_INVALID, "too many path segments"); }
  bool banded = band_starts > 0;
  cudaError_t e;
  // topology
  std::vector<size_t> tb = {sizeof(int) * S * DVG_SHAPE_INFO_STRIDE, sizeof(int) * NSEG, sizeof(int) * NSEG,
                            sizeof(int) * G * DVG_GROUP_INFO_STRIDE, sizeof(int) * NGS, sizeof(int) * NT,
                            sizeof(int) * NT, banded ? sizeof(int4) * S : 0};
  e = sc->topo.ensure(carve_size(tb));
  if (e != cudaSuccess) { delete sc; return cuda_fail(e, "allocating the scene topology"); }
  char *p = reinterpret_cast<char *>(sc->topo.ptr);
  sc->shape_info = carve<int>(p, (size_t)S * DVG_SHAPE_INFO_STRIDE);
  sc->segment_ctrl = carve<int>(p, NSEG);
  sc->seg_point = carve<int>(p, NSEG);
  sc->group_info = carve<int>(p, (size_t)G * DVG_GROUP_INFO_STRIDE);
  sc->group_shapes = carve<int>(p, NGS);
  sc->smp_shape = carve<int>(p, NT);
  sc->smp_group = carve<int>(p, NT);
  if (banded) sc->shape_band = carve<int4>(p, S);
  struct Up { void *dst; const void *src; size_t n; } ups[] = {
      {sc->shape_band, shape_band.data(), banded ? sizeof(int4) * S : 0},
      {sc->shape_info, desc->shape_info, sizeof(int) * S * DVG_SHAPE_INFO_STRIDE},
      {sc->segment_ctrl, desc->segment_ctrl, sizeof(int) * NSEG},
      {sc->seg_point, seg_point.data(), sizeof(int) * NSEG},
      {sc->group_info, desc->group_info, sizeof(int) * G * DVG_GROUP_INFO_STRIDE},
      {sc->group_shapes, desc->group_shapes, sizeof(int) * NGS},
      {sc->smp_shape, smp_shape.data(), sizeof(int) * NT},
      {sc->smp_group, smp_group.data(), sizeof(int) * NT}};
  for (auto &u : ups) {
    if (u.n == 0) continue;
    e = cudaMemcpy(u.dst, u.src, u.n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { dvg_scene_destroy(sc); return cuda_fail(e, "uploading the scene topology"); }
  }
  // derived arrays
  std::vector<size_t> db = {
      sizeof(float) * 9 * G, sizeof(float4) * G, sizeof(float4) * G, sizeof(float) * G,    // c2s, boxes, radius
      sizeof(float4) * S, sizeof(float) * S,                                              // s_box, s_length
      sizeof(float4) * NSEG, sizeof(float) * NSEG, sizeof(float) * NSEG, sizeof(float) * NSEG,
      sizeof(int) * NSEG,                                                                  // seg_*
      sizeof(float) * NT, sizeof(float) * NT,                                              // smp cdf/pmf
      sizeof(int) * (T + 1), sizeof(int) * T, sizeof(int4) * G,                           // tiles
      sizeof(int) * (10 * (size_t)NSEG + 8 * (size_t)S + 8),                              // scratch
      sizeof(unsigned) * 4,
      sizeof(float2) * DVG_TREE_PTS * (size_t)NSEG, sizeof(float) * DVG_TREE_NODES * (size_t)NSEG,  // trees
      sizeof(int2) * G, sizeof(float4) * NR, sizeof(int4) * NR, sizeof(int4) * NR, sizeof(float) * NR,  // records
      sizeof(float4) * NR,
      banded ? sizeof(float2) * S : 0, banded ? sizeof(int) * S : 0, sizeof(int) * (size_t)band_starts,  // bands
      sizeof(int) * (size_t)band_entries};
  e = sc->derived.ensure(carve_size(db));
  if (e != cudaSuccess) { dvg_scene_destroy(sc); return cuda_fail(e, "allocating scene arenas"); }
  p = reinterpret_cast<char *>(sc->derived.ptr);
  sc->c2s = carve<float>(p, 9 * (size_t)G);
  sc->g_local_box = carve<float4>(p, G);
  sc->g_canvas_box = carve<float4>(p, G);
  sc->g_max_radius = carve<float>(p, G);
  sc->s_box = carve<float4>(p, S);
  sc->s_length = carve<float>(p, S);
  sc->seg_box = carve<float4>(p, NSEG);
  sc->seg_r = carve<float>(p, NSEG);
  sc->seg_pmf = carve<float>(p, NSEG);
  sc->seg_cdf = carve<float>(p, NSEG);
  sc->seg_order = carve<int>(p, NSEG);
  sc->smp_cdf = carve<float>(p, NT);
  sc->smp_pmf = carve<float>(p, NT);
  sc->tile_start = carve<int>(p, (size_t)T + 1);
  sc->tile_count = carve<int>(p, T);
  sc->g_tile_range = carve<int4>(p, G);
  sc->scratch = carve<int>(p, 10 * (size_t)NSEG + 8 * (size_t)S + 8);
  sc->err = carve<unsigned>(p, 4);
  sc->seg_tpts = carve<float2>(p, DVG_TREE_PTS * (size_t)NSEG);
  sc->seg_th = carve<float>(p, DVG_TREE_NODES * (size_t)NSEG);
  sc->g_rec = carve<int2>(p, G);
  sc->rec_box = carve<float4>(p, NR);
  sc->rec_a = carve<int4>(p, NR);
  sc->rec_b = carve<int4>(p, NR);
  sc->rec_r = carve<float>(p, NR);
  sc->rec_cbox = carve<float4>(p, NR);
  if (banded) {
    sc->band_geo = carve<float2>(p, S);
    sc->band_n = carve<int>(p, S);
    sc->band_start = carve<int>(p, (size_t)band_starts);
    sc->band_seg = carve<int>(p, (size_t)band_entries);
  }
  e = cudaMemset(sc->derived.ptr, 0, sc->derived.bytes);
  if (e != cudaSuccess) { dvg_scene_destroy(sc); return cuda_fail(e, "clearing scene arenas"); }
  size_t cap = (size_t)T * 32;
  if (cap < 65536) cap = 65536;
  e = sc->tiles.ensure(cap * 2 * sizeof(int));
  if (e != cudaSuccess) { dvg_scene_destroy(sc); return cuda_fail(e, "allocating tile lists"); }
  sc->tile_cap = (int)(sc->tiles.bytes / (2 * sizeof(int)));
  e = cudaMallocHost(&sc->h_status, 4 * sizeof(unsigned));
  if (e != cudaSuccess) { sc->h_status = nullptr; dvg_scene_destroy(sc); return cuda_fail(e, "pinned status"); }
  *out_scene = sc;
  return DVG_OK;
}

int dvg_scene_update_params(DvgScene *sc, const float *params, int num_params, void *stream) {
  dvg::clear_error();
  if (!sc) return fail(DVG_ERR_INVALID, "scene is NULL");
  if (!params) return fail(DVG_ERR_INVALID, "params is NULL");
  if (num_params != sc->d.num_params)
    return fail(DVG_ERR_INVALID, "num_params %d differs from the scene's %d", num_params, sc->d.num_params);
  DeviceGuard guard(sc->device);
  size_t bytes = (size_t)(num_params > 0 ? num_params : 1) * sizeof(float);
  cudaError_t e = sc->own_params.ensure(bytes);
  if (e != cudaSuccess) return cuda_fail(e, "allocating the parameter arena");
  if (num_params > 0)
    e = cudaMemcpyAsync(sc->own_params.ptr, params, (size_t)num_params * sizeof(float), cudaMemcpyDefault,
                        reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "copying the parameters");
  sc->has_params = true;
  return DVG_OK;
}

int dvg_scene_destroy(DvgScene *sc) {
  if (!sc) return DVG_OK;
  DeviceGuard guard(sc->device);
  sc->topo.release();
  sc->derived.release();
  sc->tiles.release();
  sc->weight.release();
  sc->samples.release();
  sc->dbg_val.release();
  sc->dbg_flag.release();
  sc->deep.release();
  sc->own_params.release();
  sc->edge.release();
  sc->hits.release();
  if (sc->h_status) cudaFreeHost(sc->h_status);
  for (auto &p : sc->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  for (auto ev : sc->event_pool) cudaEventDestroy(ev);
  delete sc;
  return DVG_OK;
}

int dvg_scene_profile(DvgScene *sc, int enable) {
  dvg::clear_error();
  if (!sc) return fail(DVG_ERR_INVALID, "scene is NULL");
  DeviceGuard guard(sc->device);
  for (auto &p : sc->pending) { sc->event_pool.push_back(p.a); sc->event_pool.push_back(p.b); }
  sc->pending.clear();
  for (int k = 0; k < 16; k++) { sc->total_ms[k] = 0; sc->launches[k] = 0; }
  sc->profiling = enable != 0;
  return DVG_OK;
}

int dvg_scene_profile_read(DvgScene *sc, DvgKernelTime *out, int max_entries, int *num_entries) {
  dvg::clear_error();
  if (!sc || !num_entries) return fail(DVG_ERR_INVALID, "scene / num_entries is NULL");
  DeviceGuard guard(sc->device);
  for (auto &p : sc->pending) {
    cudaError_t e = cudaEventSynchronize(p.b);
    if (e != cudaSuccess) return cuda_fail(e, "reading kernel timings");
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      sc->total_ms[p.kid] += ms;
      sc->launches[p.kid] += 1;
    }
    sc->event_pool.push_back(p.a);
    sc->event_pool.push_back(p.b);
  }
  sc->pending.clear();
  int n = 0;
  for (int k = 0; k < K_COUNT; k++) {
    if (sc->launches[k] == 0) continue;
    if (out && n < max_entries) {
      out[n].name = kKernelNames[k];
      out[n].launches = sc->launches[k];
      out[n].total_ms = sc->total_ms[k];
    }
    n++;
  }
  *num_entries = n;
  return DVG_OK;
}

int dvg_scene_info(const DvgScene *sc, int32_t *num_params, int32_t *device) {
  dvg::clear_error();
  if (!sc) return fail(DVG_ERR_INVALID, "scene is NULL");
  if (num_params) *num_params = sc->d.num_params;
  if (device) *device = sc->device;
  return DVG_OK;
}

int dvg_scene_sync(DvgScene *sc, void *stream) {
  dvg::clear_error();
  if (!sc) return fail(DVG_ERR_INVALID, "scene is NULL");
  DeviceGuard guard(sc->device);
  bool retry = false;
  int st = finish(sc, reinterpret_cast<cudaStream_t>(stream), &retry);
  cudaMemsetAsync(sc->err, 0, 2 * sizeof(unsigned), reinterpret_cast<cudaStream_t>(stream));
  if (st == DVG_OK && retry)
    return fail(DVG_ERR_CAPACITY, "tile candidate lists overflowed and were grown; repeat the affected calls");
  return st;
}

int dvg_render_forward(DvgScene *sc, const DvgRenderArgs *a, float *image, float *sdf, void *stream) {
  dvg::clear_error();
  DvgRenderArgs tmp;
  a = with_params(sc, a, tmp);
  int st = check_args(sc, a);
  if (st != DVG_OK) return st;
  if ((image == nullptr) == (sdf == nullptr)) return fail(DVG_ERR_INVALID, "exactly one of image / sdf must be set");
  if (image && a->num_eval_positions > 0) return fail(DVG_ERR_INVALID, "eval_positions apply to the sdf output only");
  if (image && (reinterpret_cast<uintptr_t>(image) & 15u)) return fail(DVG_ERR_INVALID, "image must be 16-byte aligned");
  DeviceGuard guard(sc->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  size_t npx = (size_t)a->width * a->height, n = npx * a->num_samples_x * a->num_samples_y;
  sc->hit_live = false;
  bool cache = image != nullptr && !(a->flags & DVG_FLAG_NO_FRAG_CACHE);
  bool pf = a->use_prefiltering != 0;
  if (image && !cache) sc->hits.release();
  cudaError_t e = sc->weight.ensure(npx * sizeof(float));
  if (e == cudaSuccess && image) e = sc->samples.ensure(n * sizeof(float4));
  if (e == cudaSuccess && cache) e = sc->hits.ensure(hit_bytes(sc, n, pf));
  // the forward defers its open fp64 walks as the boundary pass does, in the same arena
  bool defer = image && !pf && edge_defers(sc, n);
  if (e == cudaSuccess && defer) e = sc->edge.ensure(edge_bytes(sc, n));
  if (e != cudaSuccess) return cuda_fail(e, "allocating image arenas");
  if (sc->d.num_groups == 0 && image) {
    // empty scene: the background (or transparent black), unfiltered
    e = a->background ? cudaMemcpyAsync(image, a->background, npx * 4 * sizeof(float), cudaMemcpyDeviceToDevice, s)
                      : cudaMemsetAsync(image, 0, npx * 4 * sizeof(float), s);
    if (e == cudaSuccess && !(a->flags & DVG_FLAG_NO_SYNC)) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? DVG_OK : cuda_fail(e, "empty-scene forward");
  }
  for (int attempt = 0; attempt < 3; attempt++) {
    DevScene S = make_dev(sc, a->params);
    if ((st = prepare(sc, S, a, s)) != DVG_OK) return st;
    DevRender R = make_render(sc, a);
    if (image) {
      float4 *samples = reinterpret_cast<float4 *>(sc->samples.ptr);
      HitArena h{};
      if (cache) {
        h = hit_arena(sc, n, pf);
        set_hit_cache(R, h, pf);
      }
      EdgeRecords D{};
      if (defer) D = edge_records(sc, n);
      timed(sc, K_WEIGHT, s, [&] { dvg::launch_weight(S, R, s); });
      timed(sc, K_SAMPLE_FWD, s, [&] { dvg::launch_sample_fwd(S, R, samples, s, defer ? &D : nullptr); });
      timed(sc, K_RESOLVE, s, [&] { dvg::launch_resolve(R, samples, image, s); });
      e = cudaGetLastError();
      if (e == cudaSuccess && cache && sc->d.num_params > 0)
        e = cudaMemcpyAsync(h.params, a->params, (size_t)sc->d.num_params * sizeof(float), cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess && cache) {
        sc->hit_live = true;
        sc->hit_pf = pf;
        sc->hit_w = a->width;
        sc->hit_h = a->height;
        sc->hit_nsx = a->num_samples_x;
        sc->hit_nsy = a->num_samples_y;
        sc->hit_seed = a->seed;
      }
    } else {
      size_t nout = a->num_eval_positions > 0 ? (size_t)a->num_eval_positions : npx;
      e = cudaMemsetAsync(sdf, 0, nout * sizeof(float), s);
      if (e == cudaSuccess) {
        timed(sc, K_SDF, s, [&] {
          dvg::launch_sdf(S, R, a->num_eval_positions > 0 ? a->eval_positions : nullptr, a->num_eval_positions, sdf,
                          nullptr, s);
        });
        e = cudaGetLastError();
      }
    }
    if (e != cudaSuccess) return cuda_fail(e, "forward launch");
    if (a->flags & DVG_FLAG_NO_SYNC) return DVG_OK;
    bool retry = false;
    if ((st = finish(sc, s, &retry)) != DVG_OK) return st;
    if (!retry) {
      if (cache) grow_hit_chunks(sc, n, pf);
      return DVG_OK;
    }
  }
  return fail(DVG_ERR_CAPACITY, "tile candidate lists kept overflowing");
}

int dvg_render_backward(DvgScene *sc, const DvgRenderArgs *a, const float *d_image, const float *d_sdf,
                        float *d_params, float *d_background, float *d_translation, void *stream) {
  dvg::clear_error();
  DvgRenderArgs tmp;
  a = with_params(sc, a, tmp);
  int st = check_args(sc, a);
  if (st != DVG_OK) return st;
  if ((d_image == nullptr) == (d_sdf == nullptr)) return fail(DVG_ERR_INVALID, "exactly one of d_image / d_sdf must be set");
  if (!d_params) return fail(DVG_ERR_INVALID, "d_params is NULL");
  if (d_image && a->num_eval_positions > 0) return fail(DVG_ERR_INVALID, "eval_positions apply to the sdf output only");
  if ((d_image && (reinterpret_cast<uintptr_t>(d_image) & 15u)) ||
      (d_background && (reinterpret_cast<uintptr_t>(d_background) & 15u)))
    return fail(DVG_ERR_INVALID, "d_image and d_background must be 16-byte aligned");
  if (d_background && !a->background) d_background = nullptr;  // no background, no background gradient
  if (sc->d.num_groups == 0) return DVG_OK;                       // empty scene: nothing to differentiate
  DeviceGuard guard(sc->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  size_t npx = (size_t)a->width * a->height, n = npx * a->num_samples_x * a->num_samples_y;
  cudaError_t e = sc->weight.ensure(npx * sizeof(float));
  if (e == cudaSuccess && d_background) e = sc->dbg_val.ensure(n * sizeof(float4));
  if (e == cudaSuccess && d_background) e = sc->dbg_flag.ensure(n * sizeof(int));
  if (e == cudaSuccess && d_image && !a->use_prefiltering) e = sc->edge.ensure(edge_bytes(sc, n));
  if (e == cudaSuccess && d_image) e = sc->deep.ensure((n + 1) * sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "allocating image arenas");
  for (int attempt = 0; attempt < 3; attempt++) {
    DevScene S = make_dev(sc, a->params);
    if ((st = prepare(sc, S, a, s)) != DVG_OK) return st;
    DevRender R = make_render(sc, a);
    R.d_params = d_params;
    R.d_translation = d_translation;
    if (d_image) {
      R.d_image = d_image;
      R.d_background = d_background;
      R.deep_count = reinterpret_cast<int *>(sc->deep.ptr);
      R.deep_list = R.deep_count + 1;
      float4 *dbg_val = reinterpret_cast<float4 *>(sc->dbg_val.ptr);
      int *dbg_flag = reinterpret_cast<int *>(sc->dbg_flag.ptr);
      if (hit_matches(sc, a)) {
        bool pf = a->use_prefiltering != 0;
        HitArena h = hit_arena(sc, n, pf);
        e = cudaMemsetAsync(h.stale, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return cuda_fail(e, "backward launch");
        if (sc->d.num_params > 0) dvg::launch_hit_check(a->params, h.params, sc->d.num_params, h.stale, s);
        set_hit_cache(R, h, pf);
        R.hit_chunk_count = nullptr;  // read only: the backward hands out no chunks
        R.hit_stale = h.stale;
      }
      timed(sc, K_WEIGHT, s, [&] { dvg::launch_weight(S, R, s); });
      timed(sc, K_SAMPLE_BWD, s, [&] { dvg::launch_sample_bwd(S, R, dbg_val, dbg_flag, s); });
      if (d_background) timed(sc, K_BG_COMBINE, s, [&] { dvg::launch_bg_combine(S, R, dbg_val, dbg_flag, s); });
      if (!a->use_prefiltering) {
        EdgeRecords E = edge_records(sc, n);
        timed(sc, K_EDGE, s, [&] { dvg::launch_edge(S, R, E, s); });
      }
    } else {
      timed(sc, K_SDF, s, [&] {
        dvg::launch_sdf(S, R, a->num_eval_positions > 0 ? a->eval_positions : nullptr, a->num_eval_positions,
                        nullptr, d_sdf, s);
      });
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "backward launch");
    if (a->flags & DVG_FLAG_NO_SYNC) return DVG_OK;
    bool retry = false;
    if ((st = finish(sc, s, &retry)) != DVG_OK) return st;
    if (!retry) return DVG_OK;
  }
  return fail(DVG_ERR_CAPACITY, "tile candidate lists kept overflowing");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched launches: the forward samples, the interior adjoint and the
// boundary pass of many scenes, each as one persistent launch over a work
// queue of (scene, tile) items (dvg_batch_forward / dvg_batch_backward).
// The per-scene steps around them (scene preparation, weights, resolve,
// drawing and ordering the boundary samples) are launched per scene.

struct DvgBatch {
  int device = 0;
  std::vector<DvgScene *> scenes;
  bool wide = false;            // every scene stroke-heavy: the batched walks take the wide queues
  DevBuf dev;                   // BatchScene[2n], int orders and item starts, counters
  BatchScene *h_bs = nullptr;   // pinned staging of the BatchScene arrays (forward, backward)
  int *h_ints = nullptr;        // pinned staging of the orders and item starts
  BatchScene *d_fwd = nullptr, *d_bwd = nullptr;
  int *d_ints = nullptr, *d_counters = nullptr;
  size_t nints = 0;
  // the per-scene launches around the persistent ones run on these streams,
  // forked from and joined back into the caller's stream (graph-capturable)
  static constexpr int kLanes = 8;
  cudaStream_t lanes[kLanes] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kLanes] = {};
  cudaError_t fork(cudaStream_t s) {
    cudaError_t e = cudaEventRecord(fork_ev, s);
    for (int j = 0; j < kLanes && e == cudaSuccess; j++) e = cudaStreamWaitEvent(lanes[j], fork_ev, 0);
    return e;
  }
  cudaError_t join(cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < kLanes && e == cudaSuccess; j++) {
      e = cudaEventRecord(join_ev[j], lanes[j]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join_ev[j], 0);
    }
    return e;
  }
  cudaStream_t lane(int k) const { return lanes[k % kLanes]; }
};

namespace {

size_t batch_ints(int n) { return (size_t)5 * n + 4; }  // order, item starts (n + 1), edge order, pad

// the batch's arguments with NULL params replaced by the scenes' own arenas
const DvgRenderArgs *batch_args(DvgBatch *b, const DvgRenderArgs *args, std::vector<DvgRenderArgs> &own) {
  if (!b || !args) return args;
  own.assign(args, args + b->scenes.size());
  for (size_t i = 0; i < own.size(); i++) {
    DvgRenderArgs tmp;
    own[i] = *with_params(b->scenes[i], &own[i], tmp);
  }
  return own.data();
}

int batch_check(DvgBatch *b, const DvgRenderArgs *args) {
  if (!b) return fail(DVG_ERR_INVALID, "batch is NULL");
  if (!args) return fail(DVG_ERR_INVALID, "render arguments are NULL");
  for (size_t i = 0; i < b->scenes.size(); i++) {
    int st = check_args(b->scenes[i], &args[i]);
    if (st != DVG_OK) return st;
    if (args[i].use_prefiltering || args[i].background || args[i].num_eval_positions > 0)
      return fail(DVG_ERR_INVALID, "batched launches render sampled colour images without a background (scene %zu)",
                  i);
  }
  return DVG_OK;
}

// Scenes in descending order of work, and the first work item of each in
// that order (items of `spt` 32-sample chunks; 8 chunks per tile and sample
// plane).
void batch_items(const DvgRenderArgs *args, int n, int spt, int *order, int *item_start) {
  std::vector<std::pair<long long, int>> work;
  for (int i = 0; i < n; i++)
    work.push_back({(long long)args[i].width * args[i].height * args[i].num_samples_x * args[i].num_samples_y, i});
  std::stable_sort(work.begin(), work.end(), [](const std::pair<long long, int> &a, const std::pair<long long, int> &b) {
    return a.first > b.first;
  });
  int run = 0;
  for (int r = 0; r < n; r++) {
    const DvgRenderArgs &a = args[work[r].second];
    long long chunks = (long long)((a.width + DVG_TILE - 1) / DVG_TILE) * ((a.height + DVG_TILE - 1) / DVG_TILE) *
                       a.num_samples_x * a.num_samples_y * 8;
    order[r] = work[r].second;
    item_start[r] = run;
    run += (int)((chunks + spt - 1) / spt);
  }
  item_start[n] = run;
}

int batch_tuning(const DvgBatchTuning *t, int *ctas, int *spt) {
  *ctas = t && t->ctas_per_sm > 0 ? t->ctas_per_sm : 2;
  *spt = t && t->samples_per_thread > 0 ? t->samples_per_thread : 1;
  if (*ctas > 2 || *spt > 64) return fail(DVG_ERR_INVALID, "tuning: ctas_per_sm must be 1 or 2, samples_per_thread <= 64");
  return DVG_OK;
}

}  // namespace

extern "C" {

int dvg_batch_create(DvgScene *const *scenes, int num_scenes, DvgBatch **out) {
  dvg::clear_error();
  if (!out) return fail(DVG_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!scenes || num_scenes < 1 || num_scenes > DVG_BATCH_MAX)
    return fail(DVG_ERR_INVALID, "a batch holds 1 to %d scenes", DVG_BATCH_MAX);
  for (int i = 0; i < num_scenes; i++) {
    if (!scenes[i]) return fail(DVG_ERR_INVALID, "scene %d is NULL", i);
    if (scenes[i]->device != scenes[0]->device) return fail(DVG_ERR_INVALID, "the scenes of a batch share one device");
  }
  DvgBatch *b = new DvgBatch();
  b->device = scenes[0]->device;
  b->scenes.assign(scenes, scenes + num_scenes);
  b->wide = true;
  for (int i = 0; i < num_scenes; i++) b->wide = b->wide && scenes[i]->wide_queues;
  DeviceGuard guard(b->device);
  int n = num_scenes;
  b->nints = batch_ints(n);
  cudaError_t e = cudaMallocHost(&b->h_bs, 2 * n * sizeof(BatchScene));
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_ints, 2 * b->nints * sizeof(int));
  if (e == cudaSuccess) e = b->dev.ensure(carve_size({2 * n * sizeof(BatchScene), 2 * b->nints * sizeof(int), 16}));
  if (e != cudaSuccess) {
    dvg_batch_destroy(b);
    return cuda_fail(e, "allocating a batch");
  }
  for (int j = 0; j < DvgBatch::kLanes && e == cudaSuccess; j++) {
    e = cudaStreamCreateWithFlags(&b->lanes[j], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join_ev[j], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    dvg_batch_destroy(b);
    return cuda_fail(e, "creating a batch's streams");
  }
  char *p = reinterpret_cast<char *>(b->dev.ptr);
  b->d_fwd = carve<BatchScene>(p, n);
  b->d_bwd = carve<BatchScene>(p, n);
  b->d_ints = carve<int>(p, 2 * b->nints);
  b->d_counters = carve<int>(p, 4);
  *out = b;
  return DVG_OK;
}

int dvg_batch_destroy(DvgBatch *b) {
  dvg::clear_error();
  if (!b) return DVG_OK;
  DeviceGuard guard(b->device);
  if (b->h_bs) cudaFreeHost(b->h_bs);
  if (b->h_ints) cudaFreeHost(b->h_ints);
  for (int j = 0; j < DvgBatch::kLanes; j++) {
    if (b->lanes[j]) cudaStreamDestroy(b->lanes[j]);
    if (b->join_ev[j]) cudaEventDestroy(b->join_ev[j]);
  }
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  b->dev.release();
  delete b;
  return DVG_OK;
}

int dvg_batch_forward(DvgBatch *b, const DvgRenderArgs *args, float *const *images, const DvgBatchTuning *tuning,
                      void *stream) {
  dvg::clear_error();
  std::vector<DvgRenderArgs> own;
  args = batch_args(b, args, own);
  int st = batch_check(b, args);
  if (st != DVG_OK) return st;
  if (!images) return fail(DVG_ERR_INVALID, "images is NULL");
  int ctas, spt;
  if ((st = batch_tuning(tuning, &ctas, &spt)) != DVG_OK) return st;
  DeviceGuard guard(b->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int n = (int)b->scenes.size();
  cudaError_t e = cudaSuccess;
  BatchScene *hb = b->h_bs;
  std::vector<int> live;
  std::vector<DvgRenderArgs> live_args;
  for (int i = 0; i < n; i++)
    if (!images[i] || (reinterpret_cast<uintptr_t>(images[i]) & 15u))
      return fail(DVG_ERR_INVALID, "image %d must be set and 16-byte aligned", i);
  if ((e = b->fork(s)) != cudaSuccess) return cuda_fail(e, "batched forward");
  for (int i = 0; i < n; i++) {
    DvgScene *sc = b->scenes[i];
    const DvgRenderArgs *a = &args[i];
    cudaStream_t ls = b->lane(i);
    size_t npx = (size_t)a->width * a->height, ns = npx * a->num_samples_x * a->num_samples_y;
    sc->hit_live = false;
    if (sc->d.num_groups == 0) {  // empty scene: transparent black
      e = cudaMemsetAsync(images[i], 0, npx * 4 * sizeof(float), ls);
      if (e != cudaSuccess) return cuda_fail(e, "batched forward");
      continue;
    }
    e = sc->weight.ensure(npx * sizeof(float));
    bool cache = !(a->flags & DVG_FLAG_NO_FRAG_CACHE);
    if (!cache) sc->hits.release();
    if (e == cudaSuccess) e = sc->samples.ensure(ns * sizeof(float4));
    if (e == cudaSuccess && cache) e = sc->hits.ensure(hit_bytes(sc, ns, false));
    if (e != cudaSuccess) return cuda_fail(e, "allocating image arenas");
    BatchScene &bs = hb[live.size()];
    bs.S = make_dev(sc, a->params);
    DvgRenderArgs ai = *a;
    ai.flags |= DVG_FLAG_NO_SYNC;  // failures stay latched in the scene (dvg_scene_sync)
    if ((st = prepare(sc, bs.S, &ai, ls)) != DVG_OK) return st;
    bs.R = make_render(sc, a);
    if (cache) {
      HitArena h = hit_arena(sc, ns, false);
      set_hit_cache(bs.R, h, false);
      e = cudaMemsetAsync(h.chunk_count, 0, sizeof(int), ls);
      if (e != cudaSuccess) return cuda_fail(e, "batched forward");
    }
    bs.E = EdgeRecords{};
    bs.samples = reinterpret_cast<float4 *>(sc->samples.ptr);
    dvg::launch_weight(bs.S, bs.R, ls);
    live.push_back(i);
    live_args.push_back(*a);
  }
  if ((e = b->join(s)) != cudaSuccess) return cuda_fail(e, "batched forward");
  int nl = (int)live.size();
  if (nl == 0) return DVG_OK;
  int *order = b->h_ints, *item_start = b->h_ints + nl;
  batch_items(live_args.data(), nl, spt, order, item_start);
  e = cudaMemcpyAsync(b->d_fwd, hb, nl * sizeof(BatchScene), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_ints, b->h_ints, (2 * nl + 1) * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "staging a batch");
  dvg::launch_batch_sample_fwd(b->d_fwd, nl, b->d_ints, b->d_ints + nl, spt, ctas, b->d_counters, b->wide, s);
  if ((e = b->fork(s)) != cudaSuccess) return cuda_fail(e, "batched forward");
  for (int k = 0; k < nl; k++) {
    int i = live[k];
    DvgScene *sc = b->scenes[i];
    const DvgRenderArgs *a = &args[i];
    cudaStream_t ls = b->lane(k);
    size_t ns = (size_t)a->width * a->height * a->num_samples_x * a->num_samples_y;
    dvg::launch_resolve(hb[k].R, hb[k].samples, images[i], ls);
    if (a->flags & DVG_FLAG_NO_FRAG_CACHE) continue;
    HitArena h = hit_arena(sc, ns, false);
    if (sc->d.num_params > 0)
      e = cudaMemcpyAsync(h.params, a->params, (size_t)sc->d.num_params * sizeof(float), cudaMemcpyDeviceToDevice, ls);
    if (e != cudaSuccess) return cuda_fail(e, "batched forward");
    sc->hit_live = true;
    sc->hit_pf = false;
    sc->hit_w = a->width;
    sc->hit_h = a->height;
    sc->hit_nsx = a->num_samples_x;
    sc->hit_nsy = a->num_samples_y;
    sc->hit_seed = a->seed;
  }
  if ((e = b->join(s)) != cudaSuccess) return cuda_fail(e, "batched forward");
  e = cudaGetLastError();
  return e == cudaSuccess ? DVG_OK : cuda_fail(e, "batched forward launch");
}

int dvg_batch_backward(DvgBatch *b, const DvgRenderArgs *args, const float *const *d_images, float *const *d_params,
                       const DvgBatchTuning *tuning, void *stream) {
  dvg::clear_error();
  std::vector<DvgRenderArgs> own;
  args = batch_args(b, args, own);
  int st = batch_check(b, args);
  if (st != DVG_OK) return st;
  if (!d_images || !d_params) return fail(DVG_ERR_INVALID, "d_images / d_params is NULL");
  int ctas, spt;
  if ((st = batch_tuning(tuning, &ctas, &spt)) != DVG_OK) return st;
  DeviceGuard guard(b->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int n = (int)b->scenes.size();
  cudaError_t e = cudaSuccess;
  BatchScene *hb = b->h_bs + n;
  std::vector<int> live;
  std::vector<DvgRenderArgs> live_args;
  for (int i = 0; i < n; i++)
    if (!d_images[i] || !d_params[i] || (reinterpret_cast<uintptr_t>(d_images[i]) & 15u))
      return fail(DVG_ERR_INVALID, "d_image %d / d_params %d must be set, d_image 16-byte aligned", i, i);
  // per scene, on the batch's streams: preparation, weights, the boundary samples drawn and ordered
  if ((e = b->fork(s)) != cudaSuccess) return cuda_fail(e, "batched backward");
  for (int i = 0; i < n; i++) {
    DvgScene *sc = b->scenes[i];
    const DvgRenderArgs *a = &args[i];
    cudaStream_t ls = b->lane(i);
    if (sc->d.num_groups == 0) continue;  // empty scene: nothing to differentiate
    size_t npx = (size_t)a->width * a->height, ns = npx * a->num_samples_x * a->num_samples_y;
    e = sc->weight.ensure(npx * sizeof(float));
    if (e == cudaSuccess) e = sc->edge.ensure(edge_bytes(sc, ns));
    if (e == cudaSuccess) e = sc->deep.ensure((ns + 1) * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "allocating image arenas");
    BatchScene &bs = hb[live.size()];
    bs.S = make_dev(sc, a->params);
    DvgRenderArgs ai = *a;
    ai.flags |= DVG_FLAG_NO_SYNC;
    if ((st = prepare(sc, bs.S, &ai, ls)) != DVG_OK) return st;
    bs.R = make_render(sc, a);
    bs.R.d_params = d_params[i];
    bs.R.d_image = d_images[i];
    bs.R.deep_count = reinterpret_cast<int *>(sc->deep.ptr);
    bs.R.deep_list = bs.R.deep_count + 1;
    e = cudaMemsetAsync(bs.R.deep_count, 0, sizeof(int), ls);
    if (e != cudaSuccess) return cuda_fail(e, "batched backward");
    if (hit_matches(sc, a)) {
      HitArena h = hit_arena(sc, ns, false);
      e = cudaMemsetAsync(h.stale, 0, sizeof(unsigned), ls);
      if (e != cudaSuccess) return cuda_fail(e, "batched backward");
      if (sc->d.num_params > 0) dvg::launch_hit_check(a->params, h.params, sc->d.num_params, h.stale, ls);
      set_hit_cache(bs.R, h, false);
      bs.R.hit_chunk_count = nullptr;
      bs.R.hit_stale = h.stale;
    }
    bs.E = edge_records(sc, ns);
    bs.samples = nullptr;
    dvg::launch_weight(bs.S, bs.R, ls);
    dvg::launch_edge_setup(bs.S, bs.R, bs.E, ls);
    live.push_back(i);
    live_args.push_back(*a);
  }
  if ((e = b->join(s)) != cudaSuccess) return cuda_fail(e, "batched backward");
  int nl = (int)live.size();
  if (nl == 0) return DVG_OK;
  // staged ints: scene order, item starts (nl + 1), the paired-lane scenes' order
  int *ints = b->h_ints + b->nints, *d_ints = b->d_ints + b->nints;
  int *order = ints, *item_start = ints + nl, *edge_order = ints + 2 * nl + 1;
  batch_items(live_args.data(), nl, spt, order, item_start);
  // the boundary samples are evaluated together (scenes of fewer than 8
  // groups evaluate theirs per scene)
  int n_edge = 0;
  for (int r = 0; r < nl; r++) {
    int k = order[r];
    if (b->scenes[live[k]]->d.num_groups >= 8 && hb[k].E.job_a) edge_order[n_edge++] = k;
  }
  e = cudaMemcpyAsync(b->d_bwd, hb, nl * sizeof(BatchScene), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_ints, ints, (2 * nl + 1 + n_edge) * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "staging a batch");
  dvg::launch_batch_sample_bwd(b->d_bwd, nl, d_ints, d_ints + nl, spt, ctas, b->d_counters + 1, s);
  if (n_edge > 0)
    dvg::launch_batch_edge(b->d_bwd, n_edge, d_ints + 2 * nl + 1, spt, ctas, b->d_counters + 2, b->wide, s);
  if ((e = b->fork(s)) != cudaSuccess) return cuda_fail(e, "batched backward");
  for (int k = 0; k < nl; k++)
    if (!(b->scenes[live[k]]->d.num_groups >= 8 && hb[k].E.job_a))
      dvg::launch_edge_eval(hb[k].S, hb[k].R, hb[k].E, b->lane(k));
  if ((e = b->join(s)) != cudaSuccess) return cuda_fail(e, "batched backward");
  e = cudaGetLastError();
  return e == cudaSuccess ? DVG_OK : cuda_fail(e, "batched backward launch");
}

}  // extern "C"
