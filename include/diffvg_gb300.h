/*
 * diffvg_gb300 — C ABI of the GB300-native render path of diffvg.
 *
 * The library renders 2-D vector scenes (circles, ellipses, rects, paths of
 * line / quadratic / cubic segments, grouped into shape groups with constant,
 * linear-gradient or radial-gradient paint) with per-sample pcg32 jitter, a
 * pixel filter and optional analytic prefiltering, and back-propagates an
 * image gradient to every scene parameter (interior + edge-sampling terms).
 *
 * Data model.  A scene is split in two:
 *   - its TOPOLOGY (shape kinds, point / segment counts, group membership,
 *     paint kinds) is uploaded once by dvg_scene_create() and stays resident;
 *   - its PARAMETERS are one flat fp32 arena whose layout is the order in
 *     which pydiffvg's RenderFunction.serialize_scene lists its differentiable
 *     tensors (reference: pydiffvg/render_pytorch.py:22-172).  The gradient
 *     arena written by dvg_render_backward() has the same layout, so the
 *     gradient of every input tensor is a view into it.
 *
 * Per-shape parameter layout at shape_info[SHAPE_PARAM_OFF]:
 *   circle : radius, cx, cy                 (render_pytorch.py:47-50)
 *   ellipse: rx, ry, cx, cy                 (render_pytorch.py:51-56)
 *   path   : points[2*num_points]           (render_pytorch.py:57-72)
 *            + thickness[num_points] at SHAPE_THICKNESS_OFF when present
 *   rect   : pmin_x, pmin_y, pmax_x, pmax_y (render_pytorch.py:86-91)
 *   stroke width: one float at SHAPE_STROKE_WIDTH_OFF (render_pytorch.py:94-97)
 * Per-paint layout at group_info[GROUP_FILL_OFF / GROUP_STROKE_OFF]:
 *   constant: r, g, b, a
 *   linear  : begin_x, begin_y, end_x, end_y, offsets[k], stop_colors[4k]
 *   radial  : center_x, center_y, radius_x, radius_y, offsets[k], stop_colors[4k]
 * Group transform: 9 floats (row-major 3x3 shape_to_canvas) at GROUP_XFORM_OFF.
 * Filter radius: one float at filter_radius_off.
 *
 * All functions return DVG_OK (0) or a negative DvgStatus; the message of the
 * last failure on the calling thread is returned by dvg_last_error().  No
 * function aborts the process (the reference asserts / exit(1)s instead:
 * cuda_utils.h:11-16, diffvg.cpp:542,847).
 *
 * Threading: calls are stream-ordered on the caller's cudaStream_t (passed as
 * void*).  A DvgScene owns its scratch arenas, so one scene must not be used
 * by two streams at once; distinct scenes are independent.
 */
#ifndef DIFFVG_GB300_H
#define DIFFVG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shape kinds: values of diffvg.ShapeType (shape.h:9-14). */
enum DvgShapeKind { DVG_CIRCLE = 0, DVG_ELLIPSE = 1, DVG_PATH = 2, DVG_RECT = 3 };
/* Paint kinds: values of diffvg.ColorType (color.h:7-11); -1 = no paint. */
enum DvgPaintKind { DVG_PAINT_NONE = -1, DVG_CONSTANT = 0, DVG_LINEAR = 1, DVG_RADIAL = 2 };
/* Pixel filters: values of diffvg.FilterType (filter.h:6-11).  DVG_GAUSSIAN
 * has no counterpart in the reference: a separable Gaussian of standard
 * deviation radius / 2, shifted to reach 0 at the edge of its support
 * |dx|, |dy| <= radius. */
enum DvgFilterKind { DVG_BOX = 0, DVG_TENT = 1, DVG_PARABOLIC = 2, DVG_HANN = 3, DVG_GAUSSIAN = 4 };

enum DvgStatus {
  DVG_OK = 0,
  DVG_ERR_INVALID = -1,      /* malformed scene or arguments                    */
  DVG_ERR_CUDA = -2,         /* a CUDA runtime call failed                       */
  DVG_ERR_CAPACITY = -3,     /* a per-sample fragment list overflowed            */
  DVG_ERR_UNSUPPORTED = -4,  /* the reference aborts on this input (e.g. ellipse stroke) */
  DVG_ERR_SCENE = -5         /* degenerate scene (zero / NaN total boundary length) */
};

/* shape_info record (DVG_SHAPE_INFO_STRIDE int32 per shape). */
#define DVG_SHAPE_INFO_STRIDE 8
#define DVG_SHAPE_KIND 0
#define DVG_SHAPE_PARAM_OFF 1
#define DVG_SHAPE_NUM_POINTS 2
#define DVG_SHAPE_NUM_SEGMENTS 3
#define DVG_SHAPE_SEG_OFF 4          /* first entry of this path in segment_ctrl */
#define DVG_SHAPE_THICKNESS_OFF 5    /* -1 when the path has no per-point thickness */
#define DVG_SHAPE_FLAGS 6            /* bit0 is_closed, bit1 use_distance_approx */
#define DVG_SHAPE_STROKE_WIDTH_OFF 7

/* group_info record (DVG_GROUP_INFO_STRIDE int32 per shape group). */
#define DVG_GROUP_INFO_STRIDE 12
#define DVG_GROUP_NUM_SHAPES 0
#define DVG_GROUP_SHAPES_OFF 1       /* first entry of this group in group_shapes */
#define DVG_GROUP_FILL_KIND 2
#define DVG_GROUP_FILL_OFF 3
#define DVG_GROUP_FILL_STOPS 4
#define DVG_GROUP_STROKE_KIND 5
#define DVG_GROUP_STROKE_OFF 6
#define DVG_GROUP_STROKE_STOPS 7
#define DVG_GROUP_EVEN_ODD 8
#define DVG_GROUP_XFORM_OFF 9

/* Host-side description of a scene's topology (all pointers are host memory).
 * Replaces the arguments of diffvg.Scene(...) (diffvg.cpp:1777-1789,
 * scene.cpp:919-998) minus the parameter values. */
typedef struct DvgSceneDesc {
  int32_t canvas_width;
  int32_t canvas_height;
  int32_t num_shapes;
  int32_t num_groups;
  int32_t num_params;            /* floats in the parameter arena            */
  int32_t total_segments;        /* entries in segment_ctrl                  */
  int32_t total_group_shapes;    /* entries in group_shapes                  */
  int32_t filter_type;           /* DvgFilterKind                            */
  int32_t filter_radius_off;     /* parameter offset of the filter radius    */
  const int32_t *shape_info;     /* [num_shapes * DVG_SHAPE_INFO_STRIDE]     */
  const int32_t *segment_ctrl;   /* [total_segments] control points per segment: 0 line, 1 quadratic, 2 cubic */
  const int32_t *group_info;     /* [num_groups * DVG_GROUP_INFO_STRIDE]     */
  const int32_t *group_shapes;   /* [total_group_shapes] shape ids           */
} DvgSceneDesc;

/* Per-call render arguments (device pointers unless stated).
 * Mirrors the scalar arguments of diffvg.render (diffvg.cpp:1477-1492). */
typedef struct DvgRenderArgs {
  int32_t width;                 /* output image size (pixels)               */
  int32_t height;
  int32_t num_samples_x;
  int32_t num_samples_y;
  uint64_t seed;
  int32_t use_prefiltering;
  int32_t num_eval_positions;    /* >0: SDF at eval_positions instead of an image */
  const float *params;           /* [num_params] parameter arena; NULL: the
                                    scene's own (dvg_scene_update_params)     */
  const float *background;       /* [height*width*4] or NULL                 */
  const float *eval_positions;   /* [num_eval_positions*2] or NULL           */
  int32_t flags;                 /* DVG_FLAG_* bits                          */
} DvgRenderArgs;

/* DvgRenderArgs.flags.
 * DVG_FLAG_NO_SYNC: return right after enqueueing the work on the stream;
 *   device-side failures (fragment-list capacity, unsupported input, tile
 *   list overflow) are latched in the scene and reported by the next call
 *   without this flag or by dvg_scene_sync().  Without the flag every call
 *   waits for its stream, like the reference (diffvg.cpp:1639-1641).
 * DVG_FLAG_REUSE_PREP: the parameter values are those of the previous call
 *   on this scene, so the derived scene data (boxes, CDFs, tile lists) is
 *   reused instead of recomputed (the autograd backward right after its
 *   forward).
 * DVG_FLAG_NO_FRAG_CACHE: the forward keeps no per-sample fragment cache
 *   (about 110 B per sample, 1.1 KB per sample with prefiltering, plus
 *   chunks for samples deeper than 16 fragments) and frees the one the scene
 *   holds; the following backward recomputes each sample's fragment list, as
 *   the reference does (diffvg.cpp:605-705).  Same results, less memory, a
 *   slower backward. */
#define DVG_FLAG_NO_SYNC 1
#define DVG_FLAG_REUSE_PREP 2
#define DVG_FLAG_NO_FRAG_CACHE 4

typedef struct DvgScene DvgScene;

/* Uploads the topology and allocates the scene's resident arenas.
 * Replaces diffvg.Scene(...) (diffvg.cpp:1777-1789; scene.cpp:919-998). */
int dvg_scene_create(const DvgSceneDesc *desc, DvgScene **out_scene);

/* Frees a scene and its arenas.  Replaces Scene::~Scene (scene.cpp:1000-1023). */
int dvg_scene_destroy(DvgScene *scene);

/* Copies num_params floats (the parameter arena layout; host or device
 * memory) into the scene's own parameter arena, ordered on `stream`.  A
 * render call (single or batched) whose DvgRenderArgs.params is NULL reads
 * that arena.  num_params must equal the scene's.  The first call allocates
 * the arena (make it before capturing a graph); later calls only copy.
 * Replaces the reference's parameter upload: Scene's constructor copies the
 * shapes' and groups' parameters into the one buffer it owns
 * (scene.cpp:919-998), rebuilt on every RenderFunction call
 * (render_pytorch.py:366-368). */
int dvg_scene_update_params(DvgScene *scene, const float *params, int32_t num_params, void *stream);

/* Forward render.  Exactly one of image / sdf is non-NULL:
 *   image: [height*width*4] colour output (OutputType.color)
 *   sdf  : [height*width] or [num_eval_positions] signed distance (OutputType.sdf)
 * Replaces diffvg.render(...) called with render_image / render_sdf
 * (diffvg.cpp:1477-1649; render_pytorch.py:394-409). */
int dvg_render_forward(DvgScene *scene, const DvgRenderArgs *args,
                       float *image, float *sdf, void *stream);

/* Backward render: accumulates (+=) the gradient of <d_image, image> (or of
 * <d_sdf, sdf>) into d_params (same layout as params), d_background
 * ([height*width*4] or NULL) and d_translation ([height*width*2] or NULL).
 * The caller zeroes the outputs.  Replaces diffvg.render(...) called with
 * d_render_image / d_render_sdf / d_translation (diffvg.cpp:1477-1649;
 * render_pytorch.py:692-707 and 633-650) plus the gradient read-back of
 * Scene::get_d_shape / get_d_shape_group / get_d_filter_radius
 * (scene.cpp:1025-1035). */
int dvg_render_backward(DvgScene *scene, const DvgRenderArgs *args,
                        const float *d_image, const float *d_sdf,
                        float *d_params, float *d_background,
                        float *d_translation, void *stream);

/* Waits for `stream` and reports any failure latched by calls made with
 * DVG_FLAG_NO_SYNC since the last check; clears the latch.  A tile-list
 * overflow grows the lists and returns DVG_ERR_CAPACITY: the affected calls
 * produced no gradient and must be repeated.  No reference counterpart (the
 * reference is synchronous). */
int dvg_scene_sync(DvgScene *scene, void *stream);

/* Sizes a caller allocates for a scene: the floats of its parameter arena
 * (and of the gradient arena dvg_render_backward writes) and its device.
 * Either pointer may be NULL.  No reference counterpart (the reference's
 * Scene owns its gradient buffers). */
int dvg_scene_info(const DvgScene *scene, int32_t *num_params, int32_t *device);

/* Per-kernel GPU time of the calls on a scene, measured with CUDA events
 * recorded on the call's stream around each kernel (no reference
 * counterpart; the reference only has a wall-clock print_timing flag,
 * render_pytorch.py:8-12).  dvg_scene_profile(scene, 1) clears the table
 * and starts recording, 0 stops; dvg_scene_profile_read() waits for the
 * recorded events and returns one entry per kernel that ran. */
typedef struct DvgKernelTime {
  const char *name;              /* prepare, weight, sample_fwd, resolve, sample_bwd, bg_combine, edge, sdf */
  int64_t launches;
  double total_ms;
} DvgKernelTime;
int dvg_scene_profile(DvgScene *scene, int enable);
int dvg_scene_profile_read(DvgScene *scene, DvgKernelTime *out, int max_entries, int *num_entries);

/* Optimisation-step kernels of the batched / served paths (no reference
 * counterpart: the reference leaves the loss and the optimiser to PyTorch on
 * the host side of each call, apps/painterly_rendering.py:146-192).
 * dvg_mse_grad: d_image = scale * (image - target) over num_pixels RGBA
 *   pixels, and *loss += sum((image - target)^2) when loss is not NULL.
 * dvg_adam_step: Adam with bias correction over n parameters; lr_scale
 *   (NULL = all ones) scales each element's step, 0 freezes it; the step
 *   count *step lives on the device and is incremented, so a CUDA graph can
 *   replay the update. */
int dvg_mse_grad(const float *image, const float *target, int64_t num_pixels, float scale, float *d_image,
                 float *loss, void *stream);
int dvg_adam_step(float *params, const float *grads, float *m, float *v, const float *lr_scale, int64_t n,
                  float lr, float beta1, float beta2, float eps, int *step, void *stream);

/* Batched launches over many scenes (no reference counterpart: the reference
 * renders one scene per call, and its batch workloads loop over scenes in
 * Python, apps/generative_models/rendering.py:46-95).  A DvgBatch groups
 * existing scene handles (1 to 256, one device).  dvg_batch_forward renders
 * every scene's colour image like dvg_render_forward, and
 * dvg_batch_backward accumulates every scene's gradient like
 * dvg_render_backward, except that the sample passes of all scenes (the
 * forward samples, the interior adjoint, the boundary pass) each run as one
 * persistent launch whose warps take (scene, tile) work items from a queue,
 * largest scenes first.  args, images, d_images and d_params hold one entry
 * per scene in batch order (device pointers in host arrays); images must be
 * 16-byte aligned; sampled colour renders only (no prefiltering, background
 * or eval positions).  Calls are stream-ordered and do not wait: failures
 * latch in each scene, read them with dvg_scene_sync().  The first call on a
 * batch sizes the scenes' arenas (it may allocate); later calls with the
 * same image sizes allocate nothing, so they can be captured in a CUDA graph.
 * tuning may be NULL (2 CTAs per SM, 1 sample per thread per item). */
typedef struct DvgBatch DvgBatch;
typedef struct DvgBatchTuning {
  int32_t ctas_per_sm;         /* resident blocks per SM of the persistent launches: 1 or 2 */
  int32_t samples_per_thread;  /* samples each thread takes per work item: 1 to 64 */
} DvgBatchTuning;
int dvg_batch_create(DvgScene *const *scenes, int num_scenes, DvgBatch **out_batch);
int dvg_batch_destroy(DvgBatch *batch);
int dvg_batch_forward(DvgBatch *batch, const DvgRenderArgs *args, float *const *images,
                      const DvgBatchTuning *tuning, void *stream);
int dvg_batch_backward(DvgBatch *batch, const DvgRenderArgs *args, const float *const *d_images,
                       float *const *d_params, const DvgBatchTuning *tuning, void *stream);

/* Forward colour render that allocates nothing (no counterpart in the
 * reference).  For callers that must not allocate device memory: a host
 * process that owns all GPU memory through its own pool and bars plugins
 * from cudaMalloc, or a loop that may not allocate once running.  Takes the
 * scene description with HOST topology arrays (as dvg_scene_create), the
 * render arguments (device parameter arena, optional device background) and
 * the device image [height*width*4]; writes the image like
 * dvg_render_forward.  All scratch (topology copy, derived scene data, tile
 * lists, weight image, per-sample colours) lives in one static 16 MiB device
 * array inside the library, held by every GPU that loads it until exit;
 * calls needing more return DVG_ERR_CAPACITY.  Group shape lists must be
 * stored in group order (as serialize_scene produces them) and cover all of
 * group_shapes.  The call waits for its stream and reports device-side
 * failures itself: with no scene handle to latch them in, DVG_FLAG_NO_SYNC
 * is rejected with DVG_ERR_INVALID.  Every call
 * shares that array: calls that overlap on the GPU race.  The first call on
 * a device looks up the array's address; make it before any stream capture. */
int dvg_render_forward_noalloc(const DvgSceneDesc *desc, const DvgRenderArgs *args, float *image, void *stream);

/* Message of the last failed call on this thread ("" if none). */
const char *dvg_last_error(void);

/* Library version string. */
const char *dvg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DIFFVG_GB300_H */
