// PyTorch operators over the C ABI (include/diffvg_gb300.h), registered as
// torch.ops.diffvg_gb300.*.  They take tensors where the C ABI takes
// pointers, check device, dtype, size and layout, and pass the caller's
// current CUDA stream; the work is the dvg_* entry point's.  RenderFunction
// reaches the kernels through them, in place of the reference's pybind11
// module functions diffvg.Scene and diffvg.render (diffvg.cpp:1477-1649,
// 1777-1789).  Each returns the entry point's DvgStatus (the Python side
// raises on it with dvg_last_error()).
#include <ATen/core/Tensor.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/library.h>

#include <cstdint>
#include <cstring>
#include <optional>
#include <tuple>
#include <vector>

#include "diffvg_gb300.h"

namespace {

DvgScene *scene_of(int64_t handle) { return reinterpret_cast<DvgScene *>(static_cast<intptr_t>(handle)); }

// the scene's parameter count and device (dvg_scene_info)
void scene_sizes(int64_t handle, int64_t &num_params, int64_t &device) {
  int32_t np = 0, dev = 0;
  TORCH_CHECK(dvg_scene_info(scene_of(handle), &np, &dev) == DVG_OK, "invalid scene handle");
  num_params = np;
  device = dev;
}
void check_device(const std::optional<at::Tensor> &t, int64_t device, const char *what) {
  TORCH_CHECK(!t.has_value() || t->get_device() == device, what, " is not on the scene's device cuda:", device);
}

// a float32, contiguous CUDA tensor with at least n elements, or (optional) none
float *floats(const at::Tensor &t, int64_t n, const char *what) {
  TORCH_CHECK(t.is_cuda(), what, " must be a CUDA tensor");
  TORCH_CHECK(t.scalar_type() == at::kFloat, what, " must be float32");
  TORCH_CHECK(t.is_contiguous(), what, " must be contiguous");
  TORCH_CHECK(n < 0 || t.numel() >= n, what, " has ", t.numel(), " elements, needs ", n);
  return t.data_ptr<float>();
}
float *floats(const std::optional<at::Tensor> &t, int64_t n, const char *what) {
  return t.has_value() ? floats(*t, n, what) : nullptr;
}

void *stream_for(const at::Tensor &t) { return c10::cuda::getCurrentCUDAStream(t.get_device()).stream(); }

// dims = {width, height, num_samples_x, num_samples_y, use_prefiltering}
DvgRenderArgs render_args(c10::IntArrayRef dims, int64_t seed, int64_t flags, const std::optional<at::Tensor> &params,
                          const std::optional<at::Tensor> &background,
                          const std::optional<at::Tensor> &eval_positions) {
  TORCH_CHECK(dims.size() == 5, "dims = [width, height, num_samples_x, num_samples_y, use_prefiltering]");
  DvgRenderArgs a;
  std::memset(&a, 0, sizeof a);
  a.width = static_cast<int32_t>(dims[0]);
  a.height = static_cast<int32_t>(dims[1]);
  a.num_samples_x = static_cast<int32_t>(dims[2]);
  a.num_samples_y = static_cast<int32_t>(dims[3]);
  a.use_prefiltering = dims[4] ? 1 : 0;
  a.seed = static_cast<uint64_t>(seed);
  a.flags = static_cast<int32_t>(flags);
  a.params = floats(params, -1, "params");
  a.background = floats(background, 4 * dims[0] * dims[1], "background");
  if (eval_positions.has_value() && eval_positions->numel() > 0) {
    a.eval_positions = floats(eval_positions, -1, "eval_positions");
    a.num_eval_positions = static_cast<int32_t>(eval_positions->numel() / 2);
  }
  return a;
}

// dims = {canvas_width, canvas_height, num_shapes, num_groups, num_params, filter_type, filter_radius_off};
// the topology arrays are int32 CPU tensors.  Returns (status, scene handle).
std::tuple<int64_t, int64_t> scene_create(const at::Tensor &shape_info, const at::Tensor &segment_ctrl,
                                          const at::Tensor &group_info, const at::Tensor &group_shapes,
                                          c10::IntArrayRef dims) {
  TORCH_CHECK(dims.size() == 7, "dims = [canvas_width, canvas_height, num_shapes, num_groups, num_params, "
                                "filter_type, filter_radius_off]");
  const at::Tensor *arrays[4] = {&shape_info, &segment_ctrl, &group_info, &group_shapes};
  for (const at::Tensor *t : arrays) {
    TORCH_CHECK(!t->is_cuda() && t->scalar_type() == at::kInt && t->is_contiguous(),
                "scene topology arrays must be contiguous int32 CPU tensors");
  }
  DvgSceneDesc d;
  std::memset(&d, 0, sizeof d);
  d.canvas_width = static_cast<int32_t>(dims[0]);
  d.canvas_height = static_cast<int32_t>(dims[1]);
  d.num_shapes = static_cast<int32_t>(dims[2]);
  d.num_groups = static_cast<int32_t>(dims[3]);
  d.num_params = static_cast<int32_t>(dims[4]);
  d.filter_type = static_cast<int32_t>(dims[5]);
  d.filter_radius_off = static_cast<int32_t>(dims[6]);
  d.total_segments = static_cast<int32_t>(segment_ctrl.numel());
  d.total_group_shapes = static_cast<int32_t>(group_shapes.numel());
  d.shape_info = shape_info.data_ptr<int32_t>();
  d.segment_ctrl = segment_ctrl.data_ptr<int32_t>();
  d.group_info = group_info.data_ptr<int32_t>();
  d.group_shapes = group_shapes.data_ptr<int32_t>();
  DvgScene *sc = nullptr;
  int st = dvg_scene_create(&d, &sc);
  return {st, static_cast<int64_t>(reinterpret_cast<intptr_t>(sc))};
}

int64_t scene_destroy(int64_t scene) { return dvg_scene_destroy(scene_of(scene)); }

int64_t render_forward(int64_t scene, const std::optional<at::Tensor> &params,
                       const std::optional<at::Tensor> &background, const std::optional<at::Tensor> &eval_positions,
                       const std::optional<at::Tensor> &image, const std::optional<at::Tensor> &sdf,
                       c10::IntArrayRef dims, int64_t seed, int64_t flags) {
  TORCH_CHECK(dims.size() == 5, "dims = [width, height, num_samples_x, num_samples_y, use_prefiltering]");
  TORCH_CHECK(image.has_value() != sdf.has_value(), "exactly one of image / sdf");
  int64_t np, dev;
  scene_sizes(scene, np, dev);
  floats(params, np, "params");
  for (const auto *t : {&params, &background, &eval_positions, &image, &sdf}) check_device(*t, dev, "a tensor");
  DvgRenderArgs a = render_args(dims, seed, flags, params, background, eval_positions);
  const at::Tensor &out = image.has_value() ? *image : *sdf;
  int64_t n = image.has_value() ? 4 * dims[0] * dims[1]
                                : (a.num_eval_positions > 0 ? a.num_eval_positions : dims[0] * dims[1]);
  float *p = floats(out, n, image.has_value() ? "image" : "sdf");
  return dvg_render_forward(scene_of(scene), &a, image.has_value() ? p : nullptr, image.has_value() ? nullptr : p,
                            stream_for(out));
}

int64_t render_backward(int64_t scene, const std::optional<at::Tensor> &params,
                        const std::optional<at::Tensor> &background, const std::optional<at::Tensor> &eval_positions,
                        const std::optional<at::Tensor> &d_image, const std::optional<at::Tensor> &d_sdf,
                        const at::Tensor &d_params, const std::optional<at::Tensor> &d_background,
                        const std::optional<at::Tensor> &d_translation, c10::IntArrayRef dims, int64_t seed,
                        int64_t flags) {
  TORCH_CHECK(dims.size() == 5, "dims = [width, height, num_samples_x, num_samples_y, use_prefiltering]");
  TORCH_CHECK(d_image.has_value() != d_sdf.has_value(), "exactly one of d_image / d_sdf");
  int64_t np, dev;
  scene_sizes(scene, np, dev);
  floats(params, np, "params");
  for (const auto *t : {&params, &background, &eval_positions, &d_image, &d_sdf, &d_background, &d_translation})
    check_device(*t, dev, "a tensor");
  check_device(d_params, dev, "d_params");
  DvgRenderArgs a = render_args(dims, seed, flags, params, background, eval_positions);
  int64_t npx = dims[0] * dims[1];
  const float *di = floats(d_image, 4 * npx, "d_image");
  const float *ds = floats(d_sdf, a.num_eval_positions > 0 ? a.num_eval_positions : npx, "d_sdf");
  float *dp = floats(d_params, np, "d_params");
  float *db = floats(d_background, 4 * npx, "d_background");
  float *dt = floats(d_translation, 2 * npx, "d_translation");
  return dvg_render_backward(scene_of(scene), &a, di, ds, dp, db, dt, stream_for(d_params));
}

int64_t scene_update_params(int64_t scene, const at::Tensor &params) {
  TORCH_CHECK(params.scalar_type() == at::kFloat && params.is_contiguous(), "params must be contiguous float32");
  int64_t np, dev;
  scene_sizes(scene, np, dev);
  TORCH_CHECK(params.numel() >= np, "params has ", params.numel(), " elements, needs ", np);
  TORCH_CHECK(!params.is_cuda() || params.get_device() == dev, "params is not on the scene's device");
  void *stream = params.is_cuda() ? stream_for(params) : nullptr;
  return dvg_scene_update_params(scene_of(scene), params.data_ptr<float>(), static_cast<int32_t>(np), stream);
}

// Views of a gradient arena, one per parameter slot: numels[i] floats at
// offsets[i], shaped by the next ndims[i] entries of dims.  The backward of
// RenderFunction hands them to autograd as the gradients of the scene's
// tensors (one C++ loop in place of a Python view per tensor).
std::vector<at::Tensor> arena_views(const at::Tensor &arena, c10::IntArrayRef offsets, c10::IntArrayRef numels,
                                    c10::IntArrayRef ndims, c10::IntArrayRef dims) {
  size_t n = offsets.size();
  TORCH_CHECK(numels.size() == n && ndims.size() == n, "offsets, numels and ndims differ in length");
  TORCH_CHECK(arena.dim() == 1 && arena.is_contiguous(), "arena must be a contiguous 1-D tensor");
  int64_t total = arena.numel();
  std::vector<at::Tensor> out;
  out.reserve(n);
  size_t d = 0;
  for (size_t i = 0; i < n; i++) {
    TORCH_CHECK(offsets[i] >= 0 && numels[i] >= 0 && offsets[i] + numels[i] <= total, "slot ", i,
                " lies outside the arena");
    TORCH_CHECK(ndims[i] >= 0 && d + static_cast<size_t>(ndims[i]) <= dims.size(), "dims holds too few entries");
    at::Tensor v = arena.narrow(0, offsets[i], numels[i]);
    if (ndims[i] != 1) v = v.view(dims.slice(d, static_cast<size_t>(ndims[i])));
    d += static_cast<size_t>(ndims[i]);
    out.push_back(std::move(v));
  }
  return out;
}

int64_t scene_sync(int64_t scene, int64_t device) {
  return dvg_scene_sync(scene_of(scene), c10::cuda::getCurrentCUDAStream(static_cast<c10::DeviceIndex>(device)).stream());
}

}  // namespace

TORCH_LIBRARY(diffvg_gb300, m) {
  m.def("scene_create(Tensor shape_info, Tensor segment_ctrl, Tensor group_info, Tensor group_shapes, int[] dims) "
        "-> (int, int)",
        &scene_create);
  m.def("scene_destroy(int scene) -> int", &scene_destroy);
  m.def("render_forward(int scene, Tensor? params, Tensor? background, Tensor? eval_positions, Tensor(a!)? image, "
        "Tensor(b!)? sdf, int[] dims, int seed, int flags) -> int",
        &render_forward);
  m.def("render_backward(int scene, Tensor? params, Tensor? background, Tensor? eval_positions, Tensor? d_image, "
        "Tensor? d_sdf, Tensor(a!) d_params, Tensor(b!)? d_background, Tensor(c!)? d_translation, int[] dims, "
        "int seed, int flags) -> int",
        &render_backward);
  m.def("scene_update_params(int scene, Tensor params) -> int", &scene_update_params);
  m.def("scene_sync(int scene, int device) -> int", &scene_sync);
  m.def("arena_views(Tensor(a -> *) arena, int[] offsets, int[] numels, int[] ndims, int[] dims) -> Tensor(a)[]",
        &arena_views);
}
