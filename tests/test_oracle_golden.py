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
