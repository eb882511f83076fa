// Forward colour render that allocates nothing.
//
// Some callers cannot allocate device memory: a host application that owns
// all GPU memory through its own pool and forbids its plugins to call
// cudaMalloc, or a real-time loop that must not allocate (cudaMalloc
// synchronises the device and can fail under memory pressure) once it is
// running.  dvg_render_forward_noalloc() serves them: the caller passes the
// scene description (host arrays, as for dvg_scene_create), the parameter
// arena and the output image; every scratch buffer of the render (the
// topology copy, the derived scene data, the tile candidate lists, the
// weight image and the per-sample colours) lives in one file-scope device
// array of DVG_STATIC_SCRATCH_BYTES, which every GPU that loads the library
// holds until the process exits.  Nothing here calls cudaMalloc, cudaFree or
// a routine that allocates, on the device or the host.
//
// The array is shared by every call: a call overwrites what the previous
// one left (the status word is cleared at the start of each call), and
// calls whose work overlaps on the GPU (two streams, or two host threads)
// race on it.  The first call on a device looks up the array's device
// address (cudaGetSymbolAddress) with that device current; make that first
// call before any stream capture.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "dvg_internal.h"

#define DVG_STATIC_SCRATCH_BYTES (16u << 20)
#define DVG_STATIC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_static_scratch[DVG_STATIC_SCRATCH_BYTES];

namespace {

std::mutex g_static_mu;
void *g_static_ptr[DVG_STATIC_MAX_DEVICES];

// Device address of g_static_scratch on the current device (set up once per
// device).  In host code the symbol itself is only a host-side stand-in.
int static_scratch(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return dvg::cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= DVG_STATIC_MAX_DEVICES) return dvg::fail(DVG_ERR_INVALID, "device index %d unsupported", dev);
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return dvg::cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return DVG_OK;
}

struct Carver {
  size_t off = 0;
  template <typename T>
  size_t take(size_t n) {
    off = (off + 255) & ~size_t(255);
    size_t at = off;
    off += sizeof(T) * (n > 0 ? n : 1);
    return at;
  }
};

// first point of each path segment, and the (group, shape) pairs of the
// boundary CDF; the description was checked to list group shapes in group
// order, so pair k of group g sits at its group_shapes index
__global__ void k_static_topology(DevScene S, int *seg_point, int *smp_shape, int *smp_group) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S.num_shapes && SI(S, i, DVG_SHAPE_KIND) == DVG_PATH) {
    int nseg = SI(S, i, DVG_SHAPE_NUM_SEGMENTS), so = SI(S, i, DVG_SHAPE_SEG_OFF), pid = 0;
    for (int k = 0; k < nseg; k++) {
      seg_point[so + k] = pid;
      pid += S.segment_ctrl[so + k] + 1;
    }
  }
  if (i < S.num_groups) {
    int nsh = GI(S, i, DVG_GROUP_NUM_SHAPES), off = GI(S, i, DVG_GROUP_SHAPES_OFF);
    for (int k = 0; k < nsh; k++) {
      smp_shape[off + k] = S.group_shapes[off + k];
      smp_group[off + k] = i;
    }
  }
}

}  // namespace

extern "C" int dvg_render_forward_noalloc(const DvgSceneDesc *desc, const DvgRenderArgs *a, float *image,
                                          void *stream) {
  dvg::clear_error();
  int st = dvg::validate_desc(desc, nullptr);
  if (st != DVG_OK) return st;
  if (!a || !image || !a->params) return dvg::fail(DVG_ERR_INVALID, "arguments, image and params must be set");
  if (a->width <= 0 || a->height <= 0 || a->num_samples_x <= 0 || a->num_samples_y <= 0)
    return dvg::fail(DVG_ERR_INVALID, "image size and sample counts must be positive");
  if (a->num_eval_positions > 0) return dvg::fail(DVG_ERR_INVALID, "eval_positions apply to the sdf output only");
  if ((reinterpret_cast<uintptr_t>(image) & 15u) || (a->background && (reinterpret_cast<uintptr_t>(a->background) & 15u)))
    return dvg::fail(DVG_ERR_INVALID, "image and background must be 16-byte aligned");
  int G = desc->num_groups, NS = desc->num_shapes, NSEG = desc->total_segments, NGS = desc->total_group_shapes;
  if (a->flags & DVG_FLAG_NO_SYNC)
    return dvg::fail(DVG_ERR_INVALID,
                     "the allocation-free render has no scene handle to latch device errors in: DVG_FLAG_NO_SYNC "
                     "is not accepted");
  {
    int run = 0;
    for (int g = 0; g < G; g++) {
      const int32_t *gi = desc->group_info + (size_t)g * DVG_GROUP_INFO_STRIDE;
      if (gi[DVG_GROUP_SHAPES_OFF] != run)
        return dvg::fail(DVG_ERR_INVALID, "the allocation-free render needs group shape lists stored in group order");
      run += gi[DVG_GROUP_NUM_SHAPES];
    }
    if (run != NGS)
      return dvg::fail(DVG_ERR_INVALID, "group shape lists cover %d entries of group_shapes, not all %d", run, NGS);
  }
  long long npx = (long long)a->width * a->height, n = npx * a->num_samples_x * a->num_samples_y;
  if (n > 0x7fffffffLL) return dvg::fail(DVG_ERR_INVALID, "more than 2^31-1 samples per call");
  int tiles_x = (desc->canvas_width + DVG_TILE - 1) / DVG_TILE, tiles_y = (desc->canvas_height + DVG_TILE - 1) / DVG_TILE;
  long long T = (long long)tiles_x * tiles_y;

  // layout of the static scratch
  Carver c;
  size_t o_shape_info = c.take<int>((size_t)NS * DVG_SHAPE_INFO_STRIDE), o_seg_ctrl = c.take<int>(NSEG),
         o_seg_point = c.take<int>(NSEG), o_group_info = c.take<int>((size_t)G * DVG_GROUP_INFO_STRIDE),
         o_group_shapes = c.take<int>(NGS), o_smp_shape = c.take<int>(NGS), o_smp_group = c.take<int>(NGS);
  size_t o_c2s = c.take<float>(9 * (size_t)G), o_glb = c.take<float4>(G), o_gcb = c.take<float4>(G),
         o_gmr = c.take<float>(G), o_sbox = c.take<float4>(NS), o_slen = c.take<float>(NS),
         o_segbox = c.take<float4>(NSEG), o_segr = c.take<float>(NSEG), o_segpmf = c.take<float>(NSEG),
         o_segcdf = c.take<float>(NSEG), o_segord = c.take<int>(NSEG), o_smpcdf = c.take<float>(NGS),
         o_smppmf = c.take<float>(NGS), o_tstart = c.take<int>((size_t)T + 1), o_tcount = c.take<int>((size_t)T),
         o_trange = c.take<int4>(G), o_scratch = c.take<int>(10 * (size_t)NSEG + 8 * (size_t)NS + 8),
         o_err = c.take<unsigned>(4), o_weight = c.take<float>((size_t)npx), o_samples = c.take<float4>((size_t)n);
  int NR = dvg::count_stroke_records(desc);
  size_t o_grec = c.take<int2>(G), o_rbox = c.take<float4>(NR), o_ra = c.take<int4>(NR), o_rb = c.take<int4>(NR),
         o_rr = c.take<float>(NR), o_rcb = c.take<float4>(NR);
  size_t o_tiles = c.take<int>(0);
  c.off = o_tiles;
  if (o_tiles + 256 * sizeof(int) > DVG_STATIC_SCRATCH_BYTES)
    return dvg::fail(DVG_ERR_CAPACITY,
                     "scene and image need %zu bytes of scratch; the allocation-free render has %u",
                     o_tiles + 256 * sizeof(int), (unsigned)DVG_STATIC_SCRATCH_BYTES);
  int tile_cap = (int)((DVG_STATIC_SCRATCH_BYTES - o_tiles) / (2 * sizeof(int)));  // tile lists and masks

  void *base_v = nullptr;
  if ((st = static_scratch(&base_v)) != DVG_OK) return st;
  char *base = static_cast<char *>(base_v);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  struct Up { size_t off; const void *src; size_t bytes; } ups[] = {
      {o_shape_info, desc->shape_info, sizeof(int) * NS * DVG_SHAPE_INFO_STRIDE},
      {o_seg_ctrl, desc->segment_ctrl, sizeof(int) * NSEG},
      {o_group_info, desc->group_info, sizeof(int) * G * DVG_GROUP_INFO_STRIDE},
      {o_group_shapes, desc->group_shapes, sizeof(int) * NGS}};
  cudaError_t e = cudaSuccess;
  for (auto &u : ups)
    if (u.bytes && e == cudaSuccess) e = cudaMemcpyAsync(base + u.off, u.src, u.bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + o_err, 0, 4 * sizeof(unsigned), s);
  // segments outside any path keep first point 0, as in the allocating path
  if (e == cudaSuccess && NSEG > 0) e = cudaMemsetAsync(base + o_seg_point, 0, sizeof(int) * NSEG, s);
  if (e != cudaSuccess) return dvg::cuda_fail(e, "staging the scene in the static scratch");

  DevScene S;
  S.W = desc->canvas_width;
  S.H = desc->canvas_height;
  S.num_shapes = NS;
  S.num_groups = G;
  S.num_segments = NSEG;
  S.num_total = NGS;
  S.shape_info = reinterpret_cast<int *>(base + o_shape_info);
  S.segment_ctrl = reinterpret_cast<int *>(base + o_seg_ctrl);
  S.seg_point = reinterpret_cast<int *>(base + o_seg_point);
  S.group_info = reinterpret_cast<int *>(base + o_group_info);
  S.group_shapes = reinterpret_cast<int *>(base + o_group_shapes);
  S.smp_shape = reinterpret_cast<int *>(base + o_smp_shape);
  S.smp_group = reinterpret_cast<int *>(base + o_smp_group);
  S.P = a->params;
  S.c2s = reinterpret_cast<float *>(base + o_c2s);
  S.g_local_box = reinterpret_cast<float4 *>(base + o_glb);
  S.g_canvas_box = reinterpret_cast<float4 *>(base + o_gcb);
  S.g_max_radius = reinterpret_cast<float *>(base + o_gmr);
  S.s_box = reinterpret_cast<float4 *>(base + o_sbox);
  S.s_length = reinterpret_cast<float *>(base + o_slen);
  S.seg_box = reinterpret_cast<float4 *>(base + o_segbox);
  S.seg_r = reinterpret_cast<float *>(base + o_segr);
  S.seg_pmf = reinterpret_cast<float *>(base + o_segpmf);
  S.seg_cdf = reinterpret_cast<float *>(base + o_segcdf);
  S.seg_order = reinterpret_cast<int *>(base + o_segord);
  S.smp_cdf = reinterpret_cast<float *>(base + o_smpcdf);
  S.smp_pmf = reinterpret_cast<float *>(base + o_smppmf);
  S.tiles_x = tiles_x;
  S.tiles_y = tiles_y;
  S.tile_start = reinterpret_cast<int *>(base + o_tstart);
  S.tile_list = reinterpret_cast<int *>(base + o_tiles);
  S.tile_mask = reinterpret_cast<unsigned *>(base + o_tiles) + tile_cap;
  S.scratch = reinterpret_cast<int *>(base + o_scratch);
  S.err = reinterpret_cast<unsigned *>(base + o_err);
  S.g_rec = reinterpret_cast<int2 *>(base + o_grec);
  S.rec_box = reinterpret_cast<float4 *>(base + o_rbox);
  S.rec_a = reinterpret_cast<int4 *>(base + o_ra);
  S.rec_b = reinterpret_cast<int4 *>(base + o_rb);
  S.rec_r = reinterpret_cast<float *>(base + o_rr);
  S.rec_cbox = reinterpret_cast<float4 *>(base + o_rcb);

  if (G == 0) {
    e = a->background ? cudaMemcpyAsync(image, a->background, (size_t)npx * 4 * sizeof(float), cudaMemcpyDeviceToDevice, s)
                      : cudaMemsetAsync(image, 0, (size_t)npx * 4 * sizeof(float), s);
  } else {
    int m = NS > G ? NS : G;
    k_static_topology<<<(m + 127) / 128, 128, 0, s>>>(S, reinterpret_cast<int *>(base + o_seg_point),
                                                      reinterpret_cast<int *>(base + o_smp_shape),
                                                      reinterpret_cast<int *>(base + o_smp_group));
    e = dvg::launch_prepare(S, tile_cap, reinterpret_cast<int *>(base + o_err) + 1,
                            reinterpret_cast<int4 *>(base + o_trange), reinterpret_cast<int *>(base + o_tcount), s);
    if (e == cudaSuccess) {
      DevRender R;
      R.w = a->width;
      R.h = a->height;
      R.nsx = a->num_samples_x;
      R.nsy = a->num_samples_y;
      R.spp = R.nsx * R.nsy;
      R.seed = a->seed;
      R.prefilter = a->use_prefiltering ? 1 : 0;
      R.ftype = desc->filter_type;
      R.fr_ptr = a->params + desc->filter_radius_off;
      R.fr = 0.f;
      R.ri = 0;
      R.background = a->background;
      R.weight = reinterpret_cast<float *>(base + o_weight);
      R.d_image = nullptr;
      R.d_params = nullptr;
      R.d_background = nullptr;
      R.d_translation = nullptr;
      R.filter_radius_off = desc->filter_radius_off;
      float4 *samples = reinterpret_cast<float4 *>(base + o_samples);
      dvg::launch_weight(S, R, s);
      dvg::launch_sample_fwd(S, R, samples, s);
      dvg::launch_resolve(R, samples, image, s);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) return dvg::cuda_fail(e, "allocation-free forward launch");
  unsigned bits = 0;
  e = cudaMemcpyAsync(&bits, base + o_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return dvg::cuda_fail(e, "allocation-free forward");
  if (bits & DVG_EFLAG_BIN_OVERFLOW)
    return dvg::fail(DVG_ERR_CAPACITY, "the tile candidate lists do not fit the static scratch (%d entries)", tile_cap);
  if (bits & (DVG_EFLAG_SCENE_ZERO | DVG_EFLAG_SCENE_NAN))
    return dvg::fail(DVG_ERR_SCENE, "The total length of the shape boundaries in the scene is zero or not a number.");
  if (bits & DVG_EFLAG_FILTER) return dvg::fail(DVG_ERR_INVALID, "filter radius must be in [0, 64]");
  if (bits & DVG_EFLAG_CAPACITY)
    return dvg::fail(DVG_ERR_CAPACITY, "a sample has more fragments than the reference's per-sample limit");
  if (bits & DVG_EFLAG_UNSUPPORTED) return dvg::fail(DVG_ERR_UNSUPPORTED, "unsupported input (the reference asserts on it)");
  return DVG_OK;
}
