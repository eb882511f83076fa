"""The allocation-free forward render (dvg_render_forward_noalloc).

It is meant for callers that cannot allocate device memory, such as a host
process that owns every GPU buffer through its own pool and does not let
plugins call cudaMalloc, or a running loop that may not allocate.  It takes
the same scene description and arguments as the regular entry points and
keeps all of its scratch in a fixed device array inside the library.  This
file checks it through the C ABI against dvg_render_forward (scene handle,
allocated scratch) on calls in a row, with the tolerance of the other
forward parity tests: sampled and prefiltered scenes, a background image and
an empty scene; and that tile lists too large for the fixed array are
reported as DVG_ERR_CAPACITY.  It is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-4


def _lib():
    from diffvg_gb300 import _native
    lib = _native.load()
    lib.dvg_render_forward_noalloc.argtypes = [ctypes.POINTER(_native.SceneDesc), ctypes.POINTER(_native.RenderArgs),
                                               ctypes.c_void_p, ctypes.c_void_p]
    lib.dvg_render_forward_noalloc.restype = ctypes.c_int
    return lib


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


def _render_both(packed, params, w, h, spp, seed, background=None):
    import torch
    from diffvg_gb300 import _native
    lib = _lib()
    dev = torch.device('cuda')
    P = torch.from_numpy(np.ascontiguousarray(params, np.float32) if params.size else np.zeros(1, np.float32)).to(dev)
    bg = None if background is None else torch.from_numpy(np.ascontiguousarray(background, np.float32)).to(dev)
    args = _native.RenderArgs(w, h, spp, spp, seed, int(packed.use_prefiltering), 0, P.data_ptr(),
                              None if bg is None else bg.data_ptr(), None, 0)
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


def _packed(dvg, w, h, shapes, groups, prefilter=False):
    from diffvg_gb300.packing import pack_scene
    return pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=prefilter))


def test_noalloc_matches_allocating_forward_twice():
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    import oracle
    cases = [(workloads.stroke_scene(dvg, seed=1, num_paths=256, canvas=192), 2, 1),
             (workloads.fill_scene(dvg, seed=3, num_paths=24, canvas=160), 2, 5)]
    for (w, h, shapes, groups), spp, seed in cases:  # two calls in a row, different scenes
        packed = _packed(dvg, w, h, shapes, groups)
        out, ref = _render_both(packed, oracle.params_of(packed), w, h, spp, seed)
        assert np.abs(out - ref).max() <= FWD_TOL


def test_noalloc_prefiltered_background_and_empty_scenes():
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    import oracle
    import scenes
    # prefiltered coverage (its own sample kernel and 1 spp at pixel centres)
    w, h, shapes, groups = workloads.fill_scene(dvg, seed=4, num_paths=24, canvas=160)
    packed = _packed(dvg, w, h, shapes, groups, prefilter=True)
    out, ref = _render_both(packed, oracle.params_of(packed), w, h, 1, 2)
    assert np.abs(out - ref).max() <= FWD_TOL
    # a background image under a stroke scene
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=6, num_paths=64, canvas=96)
    packed = _packed(dvg, w, h, shapes, groups)
    bg = scenes.background_pattern(h, w)
    out, ref = _render_both(packed, oracle.params_of(packed), w, h, 2, 3, background=bg)
    assert np.abs(out - ref).max() <= FWD_TOL
    # no shape groups: the background (or transparent black) comes through
    packed = _packed(dvg, 64, 48, [], [])
    out, ref = _render_both(packed, oracle.params_of(packed), 64, 48, 2, 0, background=scenes.background_pattern(48, 64))
    assert np.abs(out - ref).max() <= FWD_TOL
    out, ref = _render_both(packed, oracle.params_of(packed), 64, 48, 2, 0)
    assert np.abs(out).max() == 0.0 and np.abs(ref).max() == 0.0


def test_noalloc_reports_tile_list_overflow():
    """256 groups that each cover a 2048 x 2048 canvas (16384 tiles) need about
    4.2 M tile-list entries, more than the fixed array holds: the call renders
    into empty lists and returns DVG_ERR_CAPACITY after its launches."""
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import _native
    lib = _lib()
    shapes, groups = [], []
    for i in range(256):
        shapes.append(dvg.Rect(p_min=torch.tensor([1.0 + i * 0.01, 1.0]), p_max=torch.tensor([2040.0, 2041.0])))
        groups.append(dvg.ShapeGroup(shape_ids=torch.tensor([i]), fill_color=torch.tensor([0.5, 0.2, 0.1, 0.3])))
    packed = _packed(dvg, 2048, 2048, shapes, groups)
    keep = []
    desc = _desc(packed, keep)
    P = packed.param_arena(torch.device('cuda'))
    out = torch.empty(16, 16, 4, device='cuda')
    args = _native.RenderArgs(16, 16, 1, 1, 0, 0, 0, P.data_ptr(), None, None, 0)
    st = lib.dvg_render_forward_noalloc(ctypes.byref(desc), ctypes.byref(args), out.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream)
    assert st == _native.DVG_ERR_CAPACITY, lib.dvg_last_error()
    assert b'tile' in lib.dvg_last_error()
    # the array is usable again by the next call
    test_noalloc_matches_allocating_forward_twice()


def test_noalloc_rejects_oversized_requests():
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import _native, workloads
    lib = _lib()
    w, h, shapes, groups = workloads.circle_scene(dvg)
    packed = _packed(dvg, w, h, shapes, groups)
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
