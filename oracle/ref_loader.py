"""TEST INFRASTRUCTURE ONLY — loads the reference implementation in-process.

Imports the reference CPU module compiled by oracle/build_ref.sh
(oracle/_ref/diffvg*.so) as `diffvg`, and the reference's own Python layer
(pydiffvg/device.py, shape.py, color.py, pixel_filter.py, render_pytorch.py
from the reference checkout) as a synthetic `pydiffvg` package.  The rest of
pydiffvg needs packages that are not installed (skimage, svgpathtools,
cssutils, matplotlib) and is not on the render path; svgpathtools is stubbed
because shape.py imports it at module level for from_svg_path only.

Used only to generate and check golden fixtures in this build container; the
GPU machine has no reference checkout, so nothing on the GPU test / bench path
imports this module.  The checkout's location comes from DVG_REFERENCE_DIR,
else from oracle/build_ref.sh (the recipe that compiles it).

variant "defined" loads the module that build_ref.sh builds with the
reference's one uninitialised read (the quintic isolator's interval slot)
given a value; one process loads one variant.
"""
import glob
import importlib.util
import os
import subprocess
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_SCRIPT = os.path.join(HERE, 'build_ref.sh')
OUT_DIRS = {'stock': '_ref', 'defined': '_ref_defined'}


def reference_dir():
    d = os.environ.get('DVG_REFERENCE_DIR')
    if d:
        return d
    return subprocess.check_output(['bash', BUILD_SCRIPT, '--print-ref-dir'], text=True).strip()


def available(ref_dir=None):
    return os.path.isfile(os.path.join(ref_dir or reference_dir(), 'diffvg.cpp'))


def build(ref_dir=None, variant='stock'):
    env = dict(os.environ, DVG_REFERENCE_DIR=ref_dir or reference_dir(), DVG_REF_VARIANT=variant)
    subprocess.check_call(['bash', BUILD_SCRIPT], env=env)
    libs = glob.glob(os.path.join(HERE, OUT_DIRS[variant], 'diffvg*.so'))
    if not libs:
        raise RuntimeError('reference module was not built')
    return libs[0]


_cached = None


def load(ref_dir=None, variant='stock'):
    """Returns (pydiffvg, diffvg) from the reference, CPU mode."""
    global _cached
    if _cached is not None:
        if _cached[2] != variant:
            raise RuntimeError('one reference variant per process')
        return _cached[:2]
    ref_dir = ref_dir or reference_dir()
    so = build(ref_dir, variant)
    spec = importlib.util.spec_from_file_location('diffvg', so)
    native = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(native)
    sys.modules['diffvg'] = native
    if 'svgpathtools' not in sys.modules:
        sys.modules['svgpathtools'] = types.ModuleType('svgpathtools')
    pkg = types.ModuleType('pydiffvg')
    pkg.__path__ = []
    sys.modules['pydiffvg'] = pkg
    for name in ('device', 'shape', 'pixel_filter', 'color', 'render_pytorch'):
        path = os.path.join(ref_dir, 'pydiffvg', name + '.py')
        spec = importlib.util.spec_from_file_location('pydiffvg.' + name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules['pydiffvg.' + name] = mod
        spec.loader.exec_module(mod)
        for k, v in vars(mod).items():
            if not k.startswith('__'):
                setattr(pkg, k, v)
    pkg.set_use_gpu(False)
    _cached = (pkg, native, variant)
    return pkg, native
