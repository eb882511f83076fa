"""The C ABI library: it builds, loads without a GPU, and exports every
function that include/diffvg_gb300.h declares."""
import ctypes
import os
import re

import pytest

from diffvg_gb300 import build, _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, 'include')):
        if fn.endswith('.h'):
            src = open(os.path.join(ROOT, 'include', fn)).read()
            src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
            names += re.findall(r'\b(dvg_[a-z_0-9]+)\s*\(', src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ('dvg_scene_create', 'dvg_scene_destroy', 'dvg_render_forward', 'dvg_render_backward',
              'dvg_last_error', 'dvg_version', 'dvg_scene_sync'):
        assert n in names


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for n in declared_functions():
        assert hasattr(lib, n), n
    assert set(_native.EXPORTS) <= set(declared_functions())


def test_binding_constants_match_the_header():
    """Every DVG_FLAG_* / DVG_OK / DVG_ERR_* value of the header has the same
    value in the ctypes binding."""
    src = open(os.path.join(ROOT, 'include', 'diffvg_gb300.h')).read()
    defs = dict(re.findall(r'#define\s+(DVG_(?:FLAG|ERR)_[A-Z_0-9]+|DVG_OK)\s+\(?(-?\d+)\)?', src))
    assert 'DVG_FLAG_NO_FRAG_CACHE' in defs
    for name, val in defs.items():
        if hasattr(_native, name):
            assert getattr(_native, name) == int(val), name
    for name in ('DVG_FLAG_NO_SYNC', 'DVG_FLAG_REUSE_PREP', 'DVG_FLAG_NO_FRAG_CACHE'):
        assert getattr(_native, name) == int(defs[name])


def test_version_and_error_strings_without_gpu():
    lib = _native.load()
    assert b'sm_103a' in lib.dvg_version()
    assert lib.dvg_last_error() is not None


def test_create_rejects_malformed_scene_without_touching_the_device():
    lib = _native.load()
    desc = _native.SceneDesc()
    desc.canvas_width = 0  # invalid: checked on the host before any CUDA call
    h = ctypes.c_void_p()
    st = lib.dvg_scene_create(ctypes.byref(desc), ctypes.byref(h))
    assert st == _native.DVG_ERR_INVALID
    assert b'canvas' in lib.dvg_last_error()


def _noalloc_call(packed, extra_group_shapes=0, flags=0):
    """Calls dvg_render_forward_noalloc with a description that fails a host
    check, so that it returns before any CUDA call (no GPU needed)."""
    import numpy as np
    lib = _native.load()
    lib.dvg_render_forward_noalloc.argtypes = [ctypes.POINTER(_native.SceneDesc), ctypes.POINTER(_native.RenderArgs),
                                               ctypes.c_void_p, ctypes.c_void_p]
    ip = ctypes.POINTER(ctypes.c_int32)
    gs = np.concatenate([packed.group_shapes.reshape(-1), np.zeros(extra_group_shapes)]).astype(np.int32)
    arrs = [np.ascontiguousarray(x.reshape(-1), dtype=np.int32) for x in
            (packed.shape_info, packed.segment_ctrl, packed.group_info)] + [gs]
    desc = _native.SceneDesc(packed.canvas_width, packed.canvas_height, packed.num_shapes, packed.num_groups,
                             packed.num_params, int(packed.segment_ctrl.size), int(gs.size), int(packed.filter_type),
                             int(packed.filter_radius_off), *[a.ctypes.data_as(ip) for a in arrs])
    dummy = np.zeros(64, np.float32)  # never dereferenced: the call fails on the host first
    args = _native.RenderArgs(16, 16, 1, 1, 0, 0, 0, dummy.ctypes.data, None, None, flags)
    st = lib.dvg_render_forward_noalloc(ctypes.byref(desc), ctypes.byref(args), dummy.ctypes.data, None)
    return st, lib.dvg_last_error()


def test_noalloc_host_checks_without_gpu():
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=1, num_paths=8, canvas=64)
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    # unused entries at the end of group_shapes would leave boundary pairs unset
    st, msg = _noalloc_call(packed, extra_group_shapes=3)
    assert st == _native.DVG_ERR_INVALID and b'group_shapes' in msg
    # errors found on the device could not be latched anywhere
    st, msg = _noalloc_call(packed, flags=_native.DVG_FLAG_NO_SYNC)
    assert st == _native.DVG_ERR_INVALID and b'NO_SYNC' in msg


def test_update_params_host_checks_without_gpu():
    lib = _native.load()
    x = (ctypes.c_float * 4)()
    assert lib.dvg_scene_update_params(None, x, 4, None) == _native.DVG_ERR_INVALID
    assert b'scene' in lib.dvg_last_error()


@pytest.mark.gpu
def test_scene_owned_parameters_render_like_passed_ones():
    """dvg_scene_update_params from host memory, then calls with params NULL:
    the image and the gradient equal those of calls that pass the arena."""
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.packing import pack_scene
    dev = torch.device('cuda', 0)
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=4, num_paths=48, canvas=96)
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    scene = _native.NativeScene(packed)
    arena = packed.param_arena(dev).contiguous()
    host = arena.cpu().contiguous()
    s = torch.cuda.current_stream(dev).cuda_stream
    img_a, img_b = torch.empty(h, w, 4, device=dev), torch.empty(h, w, 4, device=dev)
    scene.forward(_native.RenderArgs(w, h, 2, 2, 3, 0, 0, arena.data_ptr(), None, None, 0), image_ptr=img_a.data_ptr(),
                  stream=s)
    scene.update_params(host.data_ptr(), stream=s)
    scene.forward(_native.RenderArgs(w, h, 2, 2, 3, 0, 0, None, None, None, 0), image_ptr=img_b.data_ptr(), stream=s)
    assert torch.equal(img_a, img_b)
    d_img = torch.rand(h, w, 4, device=dev)
    ga, gb = torch.zeros(scene.num_params, device=dev), torch.zeros(scene.num_params, device=dev)
    scene.backward(_native.RenderArgs(w, h, 2, 2, 3, 0, 0, arena.data_ptr(), None, None, 0),
                   d_image_ptr=d_img.data_ptr(), d_params_ptr=ga.data_ptr(), stream=s)
    scene.backward(_native.RenderArgs(w, h, 2, 2, 3, 0, 0, None, None, None, 0), d_image_ptr=d_img.data_ptr(),
                   d_params_ptr=gb.data_ptr(), stream=s)
    assert float((ga - gb).norm()) <= 1e-5 * max(float(ga.norm()), 1e-12)
    scene.close()
