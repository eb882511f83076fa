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
