"""The oracle's gradients against finite differences of its own forward pass
(estimators and tolerances in fd_util): colour gradients at one seed,
circle radius and centre through the boundary term averaged over 8 seeds,
and the prefiltered coverage's vertex gradients.  CPU only."""
import fd_util

COLOR_TOL = 1e-3       # smooth at a fixed seed: one central difference
GEOMETRY_TOL = 5e-2    # 8 seeds, quarter-pixel steps (observed <= 1.2 % over 6 seed sets)
PREFILTER_TOL = 1e-2   # deterministic coverage (observed 1.4e-4)


def _oracle_backend(builder):
    import diffvg_gb300 as dvg
    from diffvg_gb300.packing import pack_scene
    import oracle
    w, h, shapes, groups, pf, spp = builder(dvg)
    filt = None
    if getattr(builder, 'filter', None):
        import torch
        filt = dvg.PixelFilter(type=getattr(dvg.diffvg.FilterType, builder.filter[0]),
                               radius=torch.tensor(builder.filter[1]))
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, filter=filt, use_prefiltering=pf))
    P = oracle.params_of(packed)

    def fwd(Pv, seed):
        return oracle.render(packed, Pv, w, h, spp, spp, seed, num_threads=4)['image']

    def bwd(Pv, seed, d):
        return oracle.render(packed, Pv, w, h, spp, spp, seed, forward=False, d_image=d, num_threads=4)['d_params']
    return packed, P, fwd, bwd


def test_oracle_gradients_match_finite_differences():
    err = fd_util.run_checks(_oracle_backend)
    print(err)
    assert err['color'] <= COLOR_TOL
    assert err['geometry'] <= GEOMETRY_TOL
    assert err['prefiltered_points'] <= PREFILTER_TOL


STROKE_WIDTH_TOL = 5e-2     # 8 seeds, quarter-pixel steps
GRADIENT_PAINT_TOL = 1e-2   # smooth at a fixed seed (observed 6.9e-4)


def test_oracle_stroke_width_and_gradient_paint_match_finite_differences():
    err = fd_util.run_extra_checks(_oracle_backend)
    print(err)
    assert err['stroke_width'] <= STROKE_WIDTH_TOL
    assert err['linear_gradient'] <= GRADIENT_PAINT_TOL


PAINT_TOL = 1e-2   # paint parameters: smooth at a fixed seed, one central difference


def test_oracle_every_paint_kind_on_fills_and_strokes_matches_finite_differences():
    """Constant, linear and radial paint on a fill and on a stroke, and a
    radial-gradient stroke in a transformed group (paint parameters and stroke
    width)."""
    err = fd_util.run_paint_checks(_oracle_backend)
    print(err)
    for name, e in err.items():
        assert e <= (STROKE_WIDTH_TOL if name.endswith('width') else PAINT_TOL), (name, e)


def test_oracle_gradients_under_each_filter_match_finite_differences():
    """Colour and circle geometry gradients under the tent, Hann and
    Gaussian pixel filters (the Gaussian is not in the reference)."""
    err = fd_util.run_filter_checks(_oracle_backend)
    print(err)
    for name, e in err.items():
        assert e <= (COLOR_TOL if name.endswith('color') else GEOMETRY_TOL), (name, e)
