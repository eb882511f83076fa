"""Shared check of a renderer against the full-size workload fixtures
(tests/golden/full_*.npz, made from the reference by make_full_golden.py).

`render(packed, params, w, h, nsx, nsy, seed, d_image=None)` returns the
image ([H, W, 4]) or, with d_image, the parameter gradient.

Forward: every channel within 1e-4 of the reference's image (plus the
fixture's quantisation error, at most 7.63e-6).  Gradients: within 1e-3
relative L2 of the reference built with its uninitialised interval slot
given a value (the behaviour this project implements), and within 1e-3 of
the stock reference beyond the distance between the two reference builds
themselves (on the fill-heavy prefiltered scene the stock build's stale
stack reads move its own gradient by 1.5e-3 relative L2).  For the
single-circle MSE fixture the loss is checked too, and the gradient is that
of the loss, taken with the reference's images.
"""
import numpy as np

import golden_util as gu

FWD_TOL = 1e-4
GRAD_TOL = 1e-3


def check(name, render):
    g = gu.load_full(name)
    img = render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed)
    d = np.abs(np.asarray(img, np.float64).reshape(g.out.shape) - g.out)
    nbad = int((d > FWD_TOL + g.out_err).sum())

    def same(digest):
        r = gu.sha256_matches(img, digest)
        return 'unknown' if r is None else r
    print('%s: forward max abs %.3g (fixture quantisation %.2g); bit-identical to the reference: %s, to the reference '
          'with the interval slot defined: %s (the two reference builds differ by up to %.3g)'
          % (name, d.max(), g.out_err, same(g.out_sha256), same(g.out_defined_sha256), g.defined_vs_stock_max_abs))
    assert nbad == 0, '%s: %d channel values differ by more than %.0e, max abs %.3g' % (name, nbad, FWD_TOL, d.max())
    if g.target is not None:
        # d loss / d image of mean((image - target)^2), from the reference's images
        n = g.out.size
        d_img = ((2.0 / n) * (g.out.astype(np.float32) - g.target.astype(np.float32))).astype(np.float32)
        loss = float(((np.asarray(img, np.float64) - g.target) ** 2).mean())
        assert abs(loss - float(g.loss)) <= 1e-6 * max(1.0, abs(float(g.loss))), (loss, float(g.loss))
    else:
        import scenes
        d_img = scenes.d_image_pattern(g.height, g.width, 4)
    dp = render(g.packed, g.params, g.width, g.height, g.nsx, g.nsy, g.seed, d_image=d_img)
    err = gu.rel_l2(dp, g.d_params)
    ref_gap = 0.0
    if g.d_params_defined is not None:
        err_def = gu.rel_l2(dp, g.d_params_defined)
        ref_gap = gu.rel_l2(g.d_params_defined, g.d_params)
        print('%s: d_params rel L2 %.3g vs the reference with the slot defined, %.3g vs the stock reference '
              '(the two reference builds differ by %.3g)' % (name, err_def, err, ref_gap))
        assert err_def <= GRAD_TOL, '%s: d_params rel L2 %.3g' % (name, err_def)
    else:
        print('%s: d_params rel L2 %.3g' % (name, err))
    assert err <= GRAD_TOL + ref_gap, '%s: d_params rel L2 %.3g' % (name, err)
