"""The SVG scene reader and writer against the reference's own
(tests/golden/svg_scenes.json and svg_saved.json, made by
tests/golden/make_svg_golden.py): the reader's shape kinds and parameters,
subpath closing, arcs as cubic pieces, paints, fill rules and group
transforms within 1e-5 for every float; the writer's documents byte for
byte."""
import json
import os

import numpy as np
import pytest

import diffvg_gb300 as dvg
import svg_cases

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, 'golden', 'svg_scenes.json')) as f:
    GOLDEN = json.load(f)


def _same(a, b, where):
    if isinstance(b, dict):
        assert isinstance(a, dict) and set(a) == set(b), where
        for k in b:
            _same(a[k], b[k], where + '.' + k)
    elif isinstance(b, list) and b and isinstance(b[0], (dict, list)):
        assert isinstance(a, list) and len(a) == len(b), where
        for i, (x, y) in enumerate(zip(a, b)):
            _same(x, y, '%s[%d]' % (where, i))
    elif isinstance(b, list) and b and isinstance(b[0], float):
        assert len(a) == len(b), where
        assert np.allclose(a, b, rtol=1e-5, atol=1e-5), where
    else:
        assert a == b, where


@pytest.mark.parametrize('name', sorted(svg_cases.CASES))
def test_svg_reader_matches_the_reference(name, tmp_path):
    f = tmp_path / (name + '.svg')
    f.write_text(svg_cases.CASES[name])
    got = svg_cases.describe(*dvg.svg_to_scene(str(f)))
    _same(got, GOLDEN[name], name)


with open(os.path.join(HERE, 'golden', 'svg_saved.json')) as f:
    SAVED = json.load(f)


@pytest.mark.parametrize('name', sorted(SAVED))
def test_svg_writer_matches_the_reference(name, tmp_path):
    """save_svg writes the reference's document, byte for byte."""
    w, h, shapes, groups, gamma = svg_cases.save_scenes(dvg)[name]
    f = tmp_path / (name + '.svg')
    dvg.save_svg(str(f), w, h, shapes, groups, use_gamma=gamma)
    assert f.read_text() == SAVED[name]
