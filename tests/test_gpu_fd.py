"""The CUDA path's gradients against finite differences of its own forward
pass, with the estimators and tolerances of the oracle's test
(test_oracle_fd.py, fd_util): colour gradients at one seed, circle radius
and centre through the boundary term averaged over 8 seeds, and the
prefiltered coverage's vertex gradients."""
import pytest

import fd_util
from test_oracle_fd import COLOR_TOL, GEOMETRY_TOL, PREFILTER_TOL

pytestmark = pytest.mark.gpu


def _cuda_backend(builder):
    import diffvg_gb300 as dvg
    from diffvg_gb300.packing import pack_scene
    import oracle
    import native_util as nu
    w, h, shapes, groups, pf, spp = builder(dvg)
    filt = None
    if getattr(builder, 'filter', None):
        import torch
        filt = dvg.PixelFilter(type=getattr(dvg.diffvg.FilterType, builder.filter[0]),
                               radius=torch.tensor(builder.filter[1]))
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, filter=filt, use_prefiltering=pf))
    P = oracle.params_of(packed)

    def fwd(Pv, seed):
        return nu.render(packed, Pv, w, h, spp, spp, seed)['image']

    def bwd(Pv, seed, d):
        return nu.render(packed, Pv, w, h, spp, spp, seed, d_out=d)['d_params']
    return packed, P, fwd, bwd


def test_cuda_gradients_match_finite_differences():
    err = fd_util.run_checks(_cuda_backend)
    print(err)
    assert err['color'] <= COLOR_TOL
    assert err['geometry'] <= GEOMETRY_TOL
    assert err['prefiltered_points'] <= PREFILTER_TOL


def test_cuda_stroke_width_and_gradient_paint_match_finite_differences():
    from test_oracle_fd import STROKE_WIDTH_TOL, GRADIENT_PAINT_TOL
    err = fd_util.run_extra_checks(_cuda_backend)
    print(err)
    assert err['stroke_width'] <= STROKE_WIDTH_TOL
    assert err['linear_gradient'] <= GRADIENT_PAINT_TOL


def test_cuda_every_paint_kind_on_fills_and_strokes_matches_finite_differences():
    """Constant, linear and radial paint on a fill and on a stroke (the
    reference cannot run gradient-coloured strokes, so finite differences are
    their only check), and a radial-gradient stroke in a transformed group (paint parameters
    and stroke width)."""
    from test_oracle_fd import STROKE_WIDTH_TOL, PAINT_TOL
    err = fd_util.run_paint_checks(_cuda_backend)
    print(err)
    for name, e in err.items():
        assert e <= (STROKE_WIDTH_TOL if name.endswith('width') else PAINT_TOL), (name, e)


def test_cuda_gradients_under_each_filter_match_finite_differences():
    """Colour and circle geometry gradients under the tent, Hann and
    Gaussian pixel filters on the CUDA path."""
    err = fd_util.run_filter_checks(_cuda_backend)
    print(err)
    for name, e in err.items():
        assert e <= (COLOR_TOL if name.endswith('color') else GEOMETRY_TOL), (name, e)
