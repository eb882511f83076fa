"""The allocation-free forward render (dvg_render_forward_noalloc).

It is meant for callers that cannot allocate device memory, such as a host
process that owns every GPU buffer through its own pool and does not let
plugins call cudaMalloc, or a running loop that may not allocate.  It takes
the same scene description and arguments as the regular entry points and
keeps all of its scratch in a fixed device array inside the library.  This
file checks it through the C ABI against dvg_render_forward (scene handle,
allocated scratch) on two calls in a row, with the tolerance of the other
forward parity tests.  It is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-4


def _desc(packed, keep):
    from diffvg_gb300 import _native
    ip = ctypes.POINTER(ctypes.c_int32)
    arrs = [np.ascontiguousarray(x.reshape(-1), dtype=np.int32) for x in
            (packed.shape_info, packed.segment_ctrl, packed.group_info, packed.group_shapes)]
    arrs = [np.zeros(1, np.int32) if a.size == 0 else a for a in arrs]
    keep.extend(arrs)
    return _native.SceneDesc(packed.canvas_width, packed.canvas_height, packed.num_shapes, packed.num_groups,
                             max(packed.num_params, 1), int(packed.segment_ctrl.size), int(packed.group_shapes.size),
                             int(packed.filter_type), int(packed.filter_radius_off),
                             *[a.ctypes.data_as(ip) for a in arrs])


def _render_both(packed, params, w, h, spp, seed):
    import torch
    from diffvg_gb300 import _native
    lib = _native.load()
    lib.dvg_render_forward_noalloc.argtypes = [ctypes.POINTER(_native.SceneDesc), ctypes.POINTER(_native.RenderArgs),
                                               ctypes.c_void_p, ctypes.c_void_p]
    lib.dvg_render_forward_noalloc.restype = ctypes.c_int
    dev = torch.device('cuda')
    P = torch.from_numpy(params).to(dev)
    args = _native.RenderArgs(w, h, spp, spp, seed, int(packed.use_prefiltering), 0, P.data_ptr(), None, None, 0)
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.empty(h, w, 4, device=dev)
    _native.NativeScene(packed).forward(args, image_ptr=ref.data_ptr(), stream=stream)
    keep = []
    desc = _desc(packed, keep)
    out = torch.full((h, w, 4), -1.0, device=dev)
    st = lib.dvg_render_forward_noalloc(ctypes.byref(desc), ctypes.byref(args), out.data_ptr(), stream)
    assert st == 0, lib.dvg_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy(), ref.cpu().numpy()


def test_noalloc_matches_allocating_forward_twice():
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.packing import pack_scene
    import oracle
    cases = [(workloads.stroke_scene(dvg, seed=1, num_paths=256, canvas=192), 2, 1),
             (workloads.fill_scene(dvg, seed=3, num_paths=24, canvas=160), 2, 5)]
    for (w, h, shapes, groups), spp, seed in cases:  # two calls in a row, different scenes
        packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
        out, ref = _render_both(packed, oracle.params_of(packed), w, h, spp, seed)
        assert np.abs(out - ref).max() <= FWD_TOL


def test_noalloc_rejects_oversized_requests():
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import _native, workloads
    from diffvg_gb300.packing import pack_scene
    lib = _native.load()
    lib.dvg_render_forward_noalloc.argtypes = [ctypes.POINTER(_native.SceneDesc), ctypes.POINTER(_native.RenderArgs),
                                               ctypes.c_void_p, ctypes.c_void_p]
    w, h, shapes, groups = workloads.circle_scene(dvg)
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    keep = []
    desc = _desc(packed, keep)
    P = packed.param_arena(torch.device('cuda'))
    out = torch.empty(2048, 2048, 4, device='cuda')
    # 2048 x 2048 x 4 samples need 64 MiB of per-sample colours: rejected on the host before any launch
    args = _native.RenderArgs(2048, 2048, 2, 2, 0, 0, 0, P.data_ptr(), None, None, 0)
    st = lib.dvg_render_forward_noalloc(ctypes.byref(desc), ctypes.byref(args), out.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream)
    assert st == _native.DVG_ERR_CAPACITY
    assert b'scratch' in lib.dvg_last_error()
