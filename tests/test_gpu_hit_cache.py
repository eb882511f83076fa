"""The backward pass takes the forward pass's per-sample fragment cache only
for the parameters, image size, sample counts and seed that made it: a
backward with other parameters or another seed must match a backward on a
fresh scene handle (same results up to the order of float atomics)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _scene():
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=5, num_paths=192, canvas=160)
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    return w, h, packed


def _params(packed):
    import oracle
    return oracle.params_of(packed)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def _d_img(h, w):
    return (np.arange(h * w * 4, dtype=np.int64).reshape(h, w, 4) * 2654435761 % 13 - 6).astype(np.float32) / 32


def test_cache_matches_fresh_backward():
    import native_util as nu
    from diffvg_gb300 import _native
    w, h, packed = _scene()
    P = _params(packed)
    d = _d_img(h, w)
    fresh = nu.render(packed, P, w, h, 2, 2, 7, d_out=d)['d_params']
    sc = _native.NativeScene(packed)
    nu.render(packed, P, w, h, 2, 2, 7, scene=sc)
    cached = nu.render(packed, P, w, h, 2, 2, 7, d_out=d, scene=sc)['d_params']
    assert _rel(cached, fresh) <= TOL


def test_stale_parameters_do_not_use_the_cache():
    import native_util as nu
    from diffvg_gb300 import _native
    w, h, packed = _scene()
    P0 = _params(packed)
    rng = np.random.default_rng(0)
    P1 = P0.copy()
    P1 += rng.normal(0, 0.75, P1.shape).astype(np.float32) * (np.abs(P0) > 1.0)  # moves points, keeps colours
    d = _d_img(h, w)
    fresh = nu.render(packed, P1, w, h, 2, 2, 7, d_out=d)['d_params']
    sc = _native.NativeScene(packed)
    nu.render(packed, P0, w, h, 2, 2, 7, scene=sc)
    after_other = nu.render(packed, P1, w, h, 2, 2, 7, d_out=d, scene=sc)['d_params']
    stale = nu.render(packed, P0, w, h, 2, 2, 7, d_out=d)['d_params']
    assert _rel(stale, fresh) > 100 * TOL   # the perturbation matters
    assert _rel(after_other, fresh) <= TOL


def test_other_seed_does_not_use_the_cache():
    import native_util as nu
    from diffvg_gb300 import _native
    w, h, packed = _scene()
    P = _params(packed)
    d = _d_img(h, w)
    fresh = nu.render(packed, P, w, h, 2, 2, 9, d_out=d)['d_params']
    sc = _native.NativeScene(packed)
    nu.render(packed, P, w, h, 2, 2, 7, scene=sc)
    after_other = nu.render(packed, P, w, h, 2, 2, 9, d_out=d, scene=sc)['d_params']
    assert _rel(after_other, fresh) <= TOL


def _fill_scene(prefilter):
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.fill_scene(dvg, seed=3, num_paths=40, canvas=192)
    return w, h, pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=prefilter))


def test_prefiltered_cache_matches_fresh_and_goes_stale():
    import native_util as nu
    from diffvg_gb300 import _native
    w, h, packed = _fill_scene(True)
    P0 = _params(packed)
    P1 = P0.copy()
    P1 += np.random.default_rng(1).normal(0, 0.75, P1.shape).astype(np.float32) * (np.abs(P0) > 1.0)
    d = _d_img(h, w)
    fresh0 = nu.render(packed, P0, w, h, 1, 1, 3, d_out=d)['d_params']
    fresh1 = nu.render(packed, P1, w, h, 1, 1, 3, d_out=d)['d_params']
    sc = _native.NativeScene(packed)
    nu.render(packed, P0, w, h, 1, 1, 3, scene=sc)
    cached = nu.render(packed, P0, w, h, 1, 1, 3, d_out=d, scene=sc)['d_params']
    nu.render(packed, P0, w, h, 1, 1, 3, scene=sc)
    after_other = nu.render(packed, P1, w, h, 1, 1, 3, d_out=d, scene=sc)['d_params']
    assert _rel(cached, fresh0) <= TOL
    assert _rel(fresh0, fresh1) > 100 * TOL
    assert _rel(after_other, fresh1) <= TOL
