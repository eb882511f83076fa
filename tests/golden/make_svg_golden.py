"""Generates tests/golden/svg_scenes.json from the reference's own SVG reader.

Runs the reference's pydiffvg/parse_svg.py (its svg_to_scene and, through
pydiffvg/shape.py, its from_svg_path) on the documents of tests/svg_cases.py
and stores each parsed scene as plain lists; runs the reference's
pydiffvg/save_svg.py on the scenes of svg_cases.save_scenes and stores the
documents it writes (tests/golden/svg_saved.json).  The reference imports three
packages that are not installed here; they are stood in for:

- svgpathtools: path data is read by diffvg_gb300.svg_path, wrapped in the
  small part of svgpathtools' Path API that from_svg_path uses
  (continuous_subpaths, isclosed, remove / append, settable end points).
  The path data grammar itself is therefore shared with the code under test;
  what the fixtures pin is everything the reference does around it: subpath
  closing, arc-to-cubic conversion, styles, classes, gradients, groups and
  transforms.
- cssutils: class rules of <style> elements ('.name { ... }').
- matplotlib.colors.to_rgba: the CSS 2.1 colour keywords.

Usage (in a container that has the reference checkout):
    python tests/golden/make_svg_golden.py [reference_dir]
"""
import importlib.util
import json
import logging
import os
import re
import sys
import tempfile
import types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref_loader  # noqa: E402
from diffvg_gb300 import svg_path as sp  # noqa: E402
from diffvg_gb300.parse_svg import _NAMED  # noqa: E402
import svg_cases  # noqa: E402


class _SubPath(list):
    @property
    def start(self):
        return self[0].start

    @property
    def end(self):
        return self[-1].end

    @end.setter
    def end(self, value):
        self[-1].end = value

    def isclosed(self):
        return self[0].start == self[-1].end


class _Path(_SubPath):
    def continuous_subpaths(self):
        return [_SubPath(s) for s in sp.continuous_subpaths(list(self))]


def _install_stubs():
    spt = sys.modules.get('svgpathtools') or types.ModuleType('svgpathtools')
    spt.parse_path = lambda d: _Path(sp.parse_path(d))
    spt.Line, spt.QuadraticBezier, spt.CubicBezier, spt.Arc = sp.Line, sp.QuadraticBezier, sp.CubicBezier, sp.Arc
    sys.modules['svgpathtools'] = spt
    sys.modules['svgpathtools.parser'] = types.ModuleType('svgpathtools.parser')
    spt.parser = sys.modules['svgpathtools.parser']

    css = types.ModuleType('cssutils')

    class _Style:
        def __init__(self, body):
            self.body = body

        def getCssText(self):
            return self.body

    class _Rule:
        def __init__(self, sel, body):
            self.selectorText = sel.strip()
            self.style = _Style(body)

    css.parseString = lambda text: [_Rule(s, b) for s, b in re.findall(r'([^{}]+)\{([^{}]*)\}', text or '')]
    css.log = logging.getLogger('cssutils')
    sys.modules['cssutils'] = css

    mpl = types.ModuleType('matplotlib')
    colors = types.ModuleType('matplotlib.colors')

    def to_rgba(s):
        key = s.strip().lower()
        if key not in _NAMED:
            raise ValueError(s)
        return tuple(c / 255.0 for c in _NAMED[key]) + (1.0,)
    colors.to_rgba = to_rgba
    mpl.colors = colors
    sys.modules['matplotlib'] = mpl
    sys.modules['matplotlib.colors'] = colors


def load_reference_reader(ref_dir):
    pyd, _ = ref_loader.load(ref_dir)
    _install_stubs()
    path = os.path.join(ref_dir, 'pydiffvg', 'parse_svg.py')
    spec = importlib.util.spec_from_file_location('pydiffvg.parse_svg', path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules['pydiffvg.parse_svg'] = mod
    spec.loader.exec_module(mod)
    return mod


def load_reference_writer(ref_dir):
    path = os.path.join(ref_dir, 'pydiffvg', 'save_svg.py')
    spec = importlib.util.spec_from_file_location('pydiffvg.save_svg', path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules['pydiffvg.save_svg'] = mod
    spec.loader.exec_module(mod)
    return mod


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else ref_loader.reference_dir()
    reader = load_reference_reader(ref)
    writer = load_reference_writer(ref)
    pyd = sys.modules['pydiffvg']
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, text in svg_cases.CASES.items():
            f = os.path.join(d, name + '.svg')
            with open(f, 'w') as fh:
                fh.write(text)
            out[name] = svg_cases.describe(*reader.svg_to_scene(f))
        saved = {}
        for name, (w, h, shapes, groups, gamma) in svg_cases.save_scenes(pyd).items():
            f = os.path.join(d, 'saved_' + name + '.svg')
            writer.save_svg(f, w, h, shapes, groups, use_gamma=gamma)
            with open(f) as fh:
                saved[name] = fh.read()
    path = os.path.join(HERE, 'svg_scenes.json')
    with open(path, 'w') as fh:
        json.dump(out, fh, indent=1)
    print('%s: %d scenes, %d bytes' % (path, len(out), os.path.getsize(path)))
    path = os.path.join(HERE, 'svg_saved.json')
    with open(path, 'w') as fh:
        json.dump(saved, fh, indent=1)
    print('%s: %d documents, %d bytes' % (path, len(saved), os.path.getsize(path)))


if __name__ == '__main__':
    main()
