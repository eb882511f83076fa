"""Bindings of libdiffvg_gb300.so (include/diffvg_gb300.h): the PyTorch
operators of libdvg_torch.so (torch.ops.diffvg_gb300, csrc/dvg_torch.cpp),
which take tensors and the current CUDA stream, and a ctypes binding of the
same C ABI for the pointer-level calls (batches, serving slots, the C-ABI
measurements and tests).

The library is the only implementation of the render path: there is no CPU
fallback, and loading fails loudly when the library is missing or when no
CUDA device is present.
"""
import ctypes
import os
import threading

import numpy as np

from . import build as _build

_FP = ctypes.POINTER(ctypes.c_float)
_IP = ctypes.POINTER(ctypes.c_int32)

DVG_OK = 0
DVG_ERR_INVALID = -1
DVG_ERR_CUDA = -2
DVG_ERR_CAPACITY = -3
DVG_ERR_UNSUPPORTED = -4
DVG_ERR_SCENE = -5

DVG_FLAG_NO_SYNC = 1
DVG_FLAG_REUSE_PREP = 2
DVG_FLAG_NO_FRAG_CACHE = 4

EXPORTS = ('dvg_scene_create', 'dvg_scene_destroy', 'dvg_scene_update_params', 'dvg_render_forward',
           'dvg_render_backward',
           'dvg_scene_sync', 'dvg_scene_info', 'dvg_scene_profile', 'dvg_scene_profile_read', 'dvg_mse_grad', 'dvg_adam_step',
           'dvg_batch_create', 'dvg_batch_destroy', 'dvg_batch_forward', 'dvg_batch_backward',
           'dvg_last_error', 'dvg_version')


class KernelTime(ctypes.Structure):
    _fields_ = [('name', ctypes.c_char_p), ('launches', ctypes.c_int64), ('total_ms', ctypes.c_double)]


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ('canvas_width', ctypes.c_int32), ('canvas_height', ctypes.c_int32),
        ('num_shapes', ctypes.c_int32), ('num_groups', ctypes.c_int32),
        ('num_params', ctypes.c_int32), ('total_segments', ctypes.c_int32),
        ('total_group_shapes', ctypes.c_int32), ('filter_type', ctypes.c_int32),
        ('filter_radius_off', ctypes.c_int32),
        ('shape_info', _IP), ('segment_ctrl', _IP), ('group_info', _IP), ('group_shapes', _IP),
    ]


class RenderArgs(ctypes.Structure):
    _fields_ = [
        ('width', ctypes.c_int32), ('height', ctypes.c_int32),
        ('num_samples_x', ctypes.c_int32), ('num_samples_y', ctypes.c_int32),
        ('seed', ctypes.c_uint64), ('use_prefiltering', ctypes.c_int32),
        ('num_eval_positions', ctypes.c_int32),
        ('params', ctypes.c_void_p), ('background', ctypes.c_void_p), ('eval_positions', ctypes.c_void_p),
        ('flags', ctypes.c_int32),
    ]


class BatchTuning(ctypes.Structure):
    _fields_ = [('ctas_per_sm', ctypes.c_int32), ('samples_per_thread', ctypes.c_int32)]


class RenderError(RuntimeError):
    """A failed call of the native library; `status` is the DvgStatus."""

    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


class SceneCapacityError(RenderError):
    pass


class UnsupportedSceneError(RenderError):
    pass


_lock = threading.Lock()
_lib = None


def library_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Loads the native library (building it first if it is missing or stale
    and nvcc is available)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError('libdiffvg_gb300.so is not built (run diffvg_gb300.build.build())')
        lib = ctypes.CDLL(path)
        lib.dvg_scene_create.argtypes = [ctypes.POINTER(SceneDesc), ctypes.POINTER(ctypes.c_void_p)]
        lib.dvg_scene_create.restype = ctypes.c_int
        lib.dvg_scene_destroy.argtypes = [ctypes.c_void_p]
        lib.dvg_scene_destroy.restype = ctypes.c_int
        lib.dvg_render_forward.argtypes = [ctypes.c_void_p, ctypes.POINTER(RenderArgs), ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p]
        lib.dvg_render_forward.restype = ctypes.c_int
        lib.dvg_render_backward.argtypes = [ctypes.c_void_p, ctypes.POINTER(RenderArgs), ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p]
        lib.dvg_render_backward.restype = ctypes.c_int
        lib.dvg_scene_sync.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.dvg_scene_sync.restype = ctypes.c_int
        lib.dvg_scene_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        lib.dvg_scene_info.restype = ctypes.c_int
        lib.dvg_scene_update_params.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
        lib.dvg_scene_update_params.restype = ctypes.c_int
        lib.dvg_scene_profile.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.dvg_scene_profile.restype = ctypes.c_int
        lib.dvg_scene_profile_read.argtypes = [ctypes.c_void_p, ctypes.POINTER(KernelTime), ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_int)]
        lib.dvg_scene_profile_read.restype = ctypes.c_int
        lib.dvg_mse_grad.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]
        lib.dvg_mse_grad.restype = ctypes.c_int
        lib.dvg_adam_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
        lib.dvg_adam_step.restype = ctypes.c_int
        lib.dvg_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        lib.dvg_batch_create.restype = ctypes.c_int
        lib.dvg_batch_destroy.argtypes = [ctypes.c_void_p]
        lib.dvg_batch_destroy.restype = ctypes.c_int
        lib.dvg_batch_forward.argtypes = [ctypes.c_void_p, ctypes.POINTER(RenderArgs), ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(BatchTuning), ctypes.c_void_p]
        lib.dvg_batch_forward.restype = ctypes.c_int
        lib.dvg_batch_backward.argtypes = [ctypes.c_void_p, ctypes.POINTER(RenderArgs), ctypes.POINTER(ctypes.c_void_p),
                                           ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(BatchTuning),
                                           ctypes.c_void_p]
        lib.dvg_batch_backward.restype = ctypes.c_int
        lib.dvg_last_error.argtypes = []
        lib.dvg_last_error.restype = ctypes.c_char_p
        lib.dvg_version.argtypes = []
        lib.dvg_version.restype = ctypes.c_char_p
        _lib = lib
        return lib


_ops = None


def ops():
    """torch.ops.diffvg_gb300: the PyTorch operators over the C ABI, loaded
    after (and linked against) libdiffvg_gb300.so."""
    global _ops
    if _ops is None:
        load()
        import torch
        with _lock:
            if _ops is None:
                if not os.path.exists(_build.TORCH_LIB_PATH):
                    raise RuntimeError('libdvg_torch.so is not built (run diffvg_gb300.build.build())')
                torch.ops.load_library(_build.TORCH_LIB_PATH)
                _ops = torch.ops.diffvg_gb300
    return _ops


def _i64(seed):
    """A uint64 seed as the int64 with the same bits."""
    seed = int(seed) & (2 ** 64 - 1)
    return seed - 2 ** 64 if seed >= 2 ** 63 else seed


def check(status):
    if status == DVG_OK:
        return
    msg = load().dvg_last_error().decode(errors='replace')
    if status == DVG_ERR_CAPACITY:
        raise SceneCapacityError(status, msg)
    if status == DVG_ERR_UNSUPPORTED:
        raise UnsupportedSceneError(status, msg)
    if status == DVG_ERR_INVALID:
        raise ValueError(msg)
    raise RenderError(status, msg)


class NativeScene:
    """Owns a DvgScene handle: the resident topology of a packed scene."""

    def __init__(self, packed):
        import torch
        lib = load()
        self._lib = lib
        self._ops = ops()
        arrays = [np.ascontiguousarray(x, dtype=np.int32).reshape(-1)
                  for x in (packed.shape_info, packed.segment_ctrl, packed.group_info, packed.group_shapes)]
        sizes = [int(x.size) for x in arrays]
        t = [torch.from_numpy(np.zeros(1, np.int32) if x.size == 0 else x) for x in arrays]
        if sizes[1] == 0:  # the descriptor's segment and group-shape counts are the arrays' real sizes
            t[1] = t[1][:0]
        if sizes[3] == 0:
            t[3] = t[3][:0]
        st, h = self._ops.scene_create(t[0], t[1], t[2], t[3],
                                       [packed.canvas_width, packed.canvas_height, packed.num_shapes,
                                        packed.num_groups, max(packed.num_params, 1), int(packed.filter_type),
                                        int(packed.filter_radius_off)])
        check(st)
        self.handle = ctypes.c_void_p(h)
        self.num_params = max(packed.num_params, 1)

    def close(self):
        if getattr(self, 'handle', None):
            self._lib.dvg_scene_destroy(self.handle)
            self.handle = None

    # tensor-level calls through the PyTorch operators (current CUDA stream);
    # dims = [width, height, num_samples_x, num_samples_y, use_prefiltering]
    def render_forward(self, dims, seed, flags=0, params=None, background=None, eval_positions=None, image=None,
                       sdf=None):
        check(self._ops.render_forward(self.handle.value, params, background, eval_positions, image, sdf, dims,
                                       _i64(seed), int(flags)))

    def render_backward(self, dims, seed, d_params, flags=0, params=None, background=None, eval_positions=None,
                        d_image=None, d_sdf=None, d_background=None, d_translation=None):
        check(self._ops.render_backward(self.handle.value, params, background, eval_positions, d_image, d_sdf,
                                        d_params, d_background, d_translation, dims, _i64(seed), int(flags)))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update_params(self, params_ptr, stream=0):
        """Copies the parameter arena (num_params floats at params_ptr, host
        or device memory) into the scene's own arena; calls whose
        RenderArgs.params is None then read it."""
        check(self._lib.dvg_scene_update_params(self.handle, params_ptr, self.num_params, stream))

    def forward(self, args, image_ptr=None, sdf_ptr=None, stream=0):
        check(self._lib.dvg_render_forward(self.handle, ctypes.byref(args), image_ptr, sdf_ptr, stream))

    def backward(self, args, d_image_ptr=None, d_sdf_ptr=None, d_params_ptr=None, d_background_ptr=None,
                 d_translation_ptr=None, stream=0):
        check(self._lib.dvg_render_backward(self.handle, ctypes.byref(args), d_image_ptr, d_sdf_ptr, d_params_ptr,
                                            d_background_ptr, d_translation_ptr, stream))

    def sync(self, stream=0):
        check(self._lib.dvg_scene_sync(self.handle, stream))

    def profile(self, enable):
        """Starts (clearing the table) or stops per-kernel CUDA-event timing."""
        check(self._lib.dvg_scene_profile(self.handle, 1 if enable else 0))

    def profile_read(self):
        """{kernel name: (launches, total milliseconds)} since profile(True)."""
        arr = (KernelTime * 16)()
        n = ctypes.c_int()
        check(self._lib.dvg_scene_profile_read(self.handle, arr, 16, ctypes.byref(n)))
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(min(n.value, 16))}


class NativeBatch:
    """Owns a DvgBatch handle over NativeScene objects (kept alive here):
    persistent batched launches of their sample passes."""

    def __init__(self, scenes):
        lib = load()
        self._lib = lib
        self.scenes = list(scenes)
        arr = (ctypes.c_void_p * len(self.scenes))(*[sc.handle.value for sc in self.scenes])
        h = ctypes.c_void_p()
        check(lib.dvg_batch_create(arr, len(self.scenes), ctypes.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, 'handle', None):
            self._lib.dvg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _ptrs(ptrs):
        return (ctypes.c_void_p * len(ptrs))(*ptrs)

    def forward(self, args, image_ptrs, tuning=None, stream=0):
        a = (RenderArgs * len(args))(*args)
        check(self._lib.dvg_batch_forward(self.handle, a, self._ptrs(image_ptrs),
                                          None if tuning is None else ctypes.byref(tuning), stream))

    def backward(self, args, d_image_ptrs, d_params_ptrs, tuning=None, stream=0):
        a = (RenderArgs * len(args))(*args)
        check(self._lib.dvg_batch_backward(self.handle, a, self._ptrs(d_image_ptrs), self._ptrs(d_params_ptrs),
                                           None if tuning is None else ctypes.byref(tuning), stream))


def mse_grad(image, target, d_image, loss=None, scale=None, stream=0):
    """d_image = scale * (image - target) (scale defaults to 2 / numel, the
    gradient of the mean squared error); loss += sum of squared differences."""
    n = image.numel() // 4
    if scale is None:
        scale = 2.0 / image.numel()
    check(load().dvg_mse_grad(image.data_ptr(), target.data_ptr(), n, float(scale), d_image.data_ptr(),
                              None if loss is None else loss.data_ptr(), stream))


def adam_step(params, grads, m, v, step, lr, betas=(0.9, 0.999), eps=1e-8, lr_scale=None, stream=0):
    """Adam update of a flat fp32 parameter tensor on the device; `step` is a
    one-element int32 device tensor holding the number of steps taken."""
    check(load().dvg_adam_step(params.data_ptr(), grads.data_ptr(), m.data_ptr(), v.data_ptr(),
                               None if lr_scale is None else lr_scale.data_ptr(), params.numel(), float(lr),
                               float(betas[0]), float(betas[1]), float(eps), step.data_ptr(), stream))
