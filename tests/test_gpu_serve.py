"""Serving loop on the GPU: a request's result is the same alone and in a mix
of concurrent requests of other sizes (within the gradient tolerance), and
requests that arrive later join running ones."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _request(seed, canvas, paths, steps):
    import diffvg_gb300 as dvg
    from diffvg_gb300 import serve, workloads
    w, h, shapes, groups = workloads.mixed_scene(dvg, seed, canvas, paths)
    args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
    tw, th, ts, tg = workloads.mixed_scene(dvg, seed + 50000, canvas, paths)
    targs = dvg.RenderFunction.serialize_scene(tw, th, ts, tg)
    target = dvg.RenderFunction.apply(tw, th, 2, 2, seed, None, *targs).detach()
    return serve.Request(args, workloads.noisy_target(target, seed), steps, seed=seed)


def test_result_alone_equals_result_in_mix():
    from diffvg_gb300 import serve
    alone = serve.Server()
    a = _request(11, 128, 40, 6)
    alone.submit(a)
    alone.run()
    mix = serve.Server()
    a2 = _request(11, 128, 40, 6)
    others = [_request(12, 256, 80, 9), _request(13, 64, 16, 3), _request(14, 192, 60, 7)]
    mix.submit(others[0])
    mix.submit(a2)
    mix.submit(others[1])
    mix.tick()
    mix.submit(others[2])          # arrives while the others run
    mix.run()
    assert all(r.finished is not None for r in [a2] + others)
    rel = (a.result - a2.result).norm() / a.result.norm()
    assert rel <= 1e-3
    assert a.losses == pytest.approx(a2.losses, rel=1e-3)
    assert a.losses[-1] < a.losses[0]   # the optimisation makes progress
    st = mix.stats()
    assert st['requests'] == 4 and st['p99_step_ms'] >= st['p50_step_ms'] > 0
