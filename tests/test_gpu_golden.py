"""The CUDA path (through the C ABI) against the reference's own outputs
(golden fixtures from the compiled reference, tests/golden/).

Tolerances: forward outputs within 1e-4 max abs per channel; gradients
within 1e-3 relative L2 (atomic accumulation order differs).
"""
import numpy as np
import pytest

import golden_util as gu

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-4
GRAD_TOL = 1e-3


@pytest.mark.parametrize('name', gu.names())
def test_cuda_matches_reference(name):
    import native_util as nu
    g = gu.load(name)
    common = dict(background=g.background, eval_positions=g.eval_positions, output_sdf=g.output_sdf)
    fwd = nu.render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed, **common)
    out = fwd['sdf'] if g.output_sdf else fwd['image']
    mx, nbad, _ = gu.image_report(out.reshape(g.out.shape), g.out, FWD_TOL)
    assert nbad == 0, '%s: forward max abs %.3g' % (name, mx)
    bwd = nu.render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed, d_out=g.d_out,
                    want_background_grad=g.background is not None, want_translation=g.d_translation is not None,
                    **common)
    err = gu.rel_l2(bwd['d_params'], g.d_params)
    assert err <= GRAD_TOL, '%s: d_params rel L2 %.3g' % (name, err)
    if g.d_background is not None:
        assert gu.rel_l2(bwd['d_background'], g.d_background) <= GRAD_TOL
    if g.d_translation is not None:
        assert gu.rel_l2(bwd['d_translation'], g.d_translation) <= GRAD_TOL
