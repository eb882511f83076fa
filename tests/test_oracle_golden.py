"""The CPU oracle against the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py from the compiled reference).

Tolerances (the same ones the CUDA path is held to): forward outputs within
1e-4 max abs per channel; gradients within 1e-3 relative L2 (the reference
accumulates with atomics in a different order).
"""
import numpy as np
import pytest

import golden_util as gu
import oracle

FWD_TOL = 1e-4
GRAD_TOL = 1e-3


@pytest.mark.parametrize('name', gu.names())
def test_oracle_matches_reference(name):
    g = gu.load(name)
    common = dict(background=g.background, eval_positions=g.eval_positions, output_sdf=g.output_sdf, num_threads=4)
    fwd = oracle.render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed, **common)
    out = fwd['sdf'] if g.output_sdf else fwd['image']
    mx, nbad, _ = gu.image_report(out.reshape(g.out.shape), g.out, FWD_TOL)
    assert nbad == 0, '%s: forward max abs %.3g' % (name, mx)
    kw = dict(common, forward=False, want_background_grad=g.background is not None)
    if g.output_sdf:
        kw['d_sdf'] = g.d_out
    else:
        kw['d_image'] = g.d_out
    bwd = oracle.render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed, **kw)
    assert gu.rel_l2(bwd['d_params'], g.d_params) <= GRAD_TOL, name
    if g.d_background is not None:
        assert gu.rel_l2(bwd['d_background'], g.d_background) <= GRAD_TOL
    if g.d_translation is not None:
        kw['want_translation'] = True
        bwd = oracle.render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed, **kw)
        assert gu.rel_l2(bwd['d_translation'], g.d_translation) <= GRAD_TOL, name


def test_counting_build_renders_the_same_and_counts():
    """The work-counting build (-DDVG_COUNT_OPS) computes what the plain build
    computes; its counts are deterministic per call, independent of the
    thread count, and the committed work counts of the single circle match a
    fresh count."""
    import json
    import os
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.circle_scene(dvg)
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    P = oracle.params_of(packed)
    plain = oracle.render(packed, P, w, h, 2, 2, 0, num_threads=2)
    a = oracle.render(packed, P, w, h, 2, 2, 0, num_threads=2, count_ops=True)
    b = oracle.render(packed, P, w, h, 2, 2, 0, num_threads=5, count_ops=True)
    assert np.array_equal(plain['image'], a['image'])
    assert a['ops'] == b['ops'] and a['ops']['render']['fp32'] > 0 and a['ops']['edge']['fp32'] == 0
    d_img = np.full((h, w, 4), 1e-3, np.float32)
    c = oracle.render(packed, P, w, h, 2, 2, 0, forward=False, d_image=d_img, num_threads=3, count_ops=True)
    assert c['ops']['edge']['fp32'] > 0 and c['ops']['resolve']['fp32'] == 0
    path = os.path.join(os.path.dirname(__file__), '..', 'baseline', 'work_counts.json')
    with open(path) as f:
        committed = json.load(f)['configs']['circle_256_2x2']['kernels']
    assert committed['sample_fwd']['fp32'] == a['ops']['render']['fp32']
    assert committed['weight']['fp32'] == a['ops']['weight']['fp32']
