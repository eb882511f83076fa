"""Batched optimisation path: graph replay equals the eager step, every
scene's gradient equals its single-scene backward, and the native Adam
update equals the textbook Adam update."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(n=6, seed0=100):
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.batch import BatchedScenes
    from diffvg_gb300.packing import pack_scene
    scenes = workloads.batched_scenes(dvg, seeds=range(seed0, seed0 + n), canvases=(64, 96, 128), path_range=(8, 64))
    args = [dvg.RenderFunction.serialize_scene(w, h, s, g) for (w, h, s, g) in scenes]
    b = BatchedScenes(args, seeds=list(range(seed0, seed0 + n)), lr=1e-2, streams=3)
    targets = []
    for i, p in enumerate(b.packed):
        tp = workloads.perturbed_target_params(p, b.scene_params(i), seed0 + i)
        targets.append(b.render(i, tp))
    b.set_targets(targets)
    return b


def test_batched_gradients_match_single_scene_backward():
    import torch
    from diffvg_gb300 import _native
    import native_util as nu
    b = _batch()
    before = b.params.clone()
    b.step_eager()
    torch.cuda.synchronize()
    for i, p in enumerate(b.packed):
        img = nu.render(p, before[b.offsets[i]:b.offsets[i] + p.num_params].cpu().numpy(), *b.sizes[i], b.nsx, b.nsy,
                        b.seeds[i])['image']
        d_img = 2.0 / img.size * (img - b.targets[i].cpu().numpy())
        ref = nu.render(p, before[b.offsets[i]:b.offsets[i] + p.num_params].cpu().numpy(), *b.sizes[i], b.nsx,
                        b.nsy, b.seeds[i], d_out=d_img)['d_params']
        mine = b.grads[b.offsets[i]:b.offsets[i] + p.num_params].cpu().numpy()
        assert np.linalg.norm(mine - ref) <= 1e-3 * max(np.linalg.norm(ref), 1e-12)


def test_graph_replay_equals_eager_steps():
    import torch
    b1, b2 = _batch(), _batch()
    for _ in range(3):
        b1.step()
        b2.step_eager()
    torch.cuda.synchronize()
    assert torch.allclose(b1.params, b2.params, rtol=1e-5, atol=1e-5)
    assert b1.loss() == pytest.approx(b2.loss(), rel=1e-5)


def test_native_adam_matches_reference_update():
    import torch
    from diffvg_gb300 import _native
    g = torch.Generator().manual_seed(0)
    p0 = torch.randn(1000, generator=g)
    grads = [torch.randn(1000, generator=g) for _ in range(4)]
    scale = (torch.rand(1000, generator=g) > 0.3).float()
    dev = torch.device('cuda')
    p, m, v = p0.to(dev), torch.zeros(1000, device=dev), torch.zeros(1000, device=dev)
    step = torch.zeros(1, dtype=torch.int32, device=dev)
    ref, mr, vr = p0.double().clone(), torch.zeros(1000, dtype=torch.float64), torch.zeros(1000, dtype=torch.float64)
    lr, b1, b2, eps = 1e-2, 0.9, 0.999, 1e-8
    for t, gr in enumerate(grads, 1):
        _native.adam_step(p, gr.to(dev), m, v, step, lr, (b1, b2), eps, lr_scale=scale.to(dev))
        gd = gr.double()
        mr = b1 * mr + (1 - b1) * gd
        vr = b2 * vr + (1 - b2) * gd * gd
        upd = lr * (mr / (1 - b1 ** t)) / ((vr / (1 - b2 ** t)).sqrt() + eps)
        ref = ref - scale.double() * upd
        mr = torch.where(scale > 0, mr, torch.zeros_like(mr))
        vr = torch.where(scale > 0, vr, torch.zeros_like(vr))
    torch.cuda.synchronize()
    assert int(step.item()) == 4
    assert torch.allclose(p.cpu().double(), ref, rtol=1e-5, atol=1e-6)


def _batch_mixed(n=6, seed0=200, fills=False):
    """Scenes of uneven size, one of them with fewer than 8 groups (its
    boundary pass runs per scene inside the batched call); with fills, one
    fill-heavy scene too (the batched walks then take the narrow queues)."""
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.batch import BatchedScenes
    scenes = workloads.batched_scenes(dvg, seeds=range(seed0, seed0 + n - 1), canvases=(64, 96, 160), path_range=(8, 96))
    scenes.append(workloads.stroke_scene(dvg, seed=seed0 + 99, num_paths=5, canvas=80))
    if fills:
        scenes.append(workloads.fill_scene(dvg, seed=seed0 + 98, num_paths=24, canvas=96))
        n += 1
    args = [dvg.RenderFunction.serialize_scene(w, h, s, g) for (w, h, s, g) in scenes]
    seeds = list(range(seed0, seed0 + n))
    b = BatchedScenes(args, seeds=seeds, lr=1e-2, streams=3)
    targets = []
    for i, p in enumerate(b.packed):
        tp = workloads.perturbed_target_params(p, b.scene_params(i), seed0 + i)
        targets.append(b.render(i, tp))
    b.set_targets(targets)
    return b


@pytest.mark.parametrize('tuning,fills', [((1, 1), False), ((2, 2), False), ((2, 5), False), ((1, 1), True)])
def test_persistent_batch_matches_per_scene_launches(tuning, fills):
    """One persistent launch per pass over all scenes (dvg_batch_forward /
    dvg_batch_backward) gives every scene the images of its own launches and
    its gradients within 1e-3 relative L2 (atomic order), also after graph
    replays of full steps."""
    import torch
    b1, b2 = _batch_mixed(fills=fills), _batch_mixed(fills=fills)
    b2.set_mode('persistent', tuning)
    b1.step_eager()
    b2.step_eager()
    torch.cuda.synchronize()
    for i in range(b1.num_scenes):
        assert torch.equal(b1.images[i], b2.images[i]), i
        o, n = b1.offsets[i], b1.packed[i].num_params
        g1, g2 = b1.grads[o:o + n], b2.grads[o:o + n]
        assert float((g1 - g2).norm()) <= 1e-3 * max(float(g1.norm()), 1e-12), i
    for _ in range(3):
        b1.step()
        b2.step()
    torch.cuda.synchronize()
    assert b2.check() is False
    assert torch.allclose(b1.params, b2.params, rtol=1e-4, atol=1e-4)
    assert b1.loss() == pytest.approx(b2.loss(), rel=1e-4)


def test_autotuner_picks_and_caches_a_candidate(tmp_path):
    import json
    import torch
    b = _batch_mixed(n=4, seed0=300)
    before = b.params.clone()
    path = tmp_path / 'tune.json'
    t = b.autotune(candidates=[('streams', (2, 1)), ('persistent', (2, 1)), ('persistent', (1, 2))], steps=2,
                   cache_path=str(path))
    assert set(t) == {'streams 2 1', 'persistent 2 1', 'persistent 1 2'} and all(v > 0 for v in t.values())
    assert torch.equal(b.params, before)  # the timing steps leave no trace
    cached = json.loads(path.read_text())[b.workload_key()]
    assert '%s %d %d' % (cached['mode'], *cached['tuning']) == min(t, key=t.get)
    b2 = _batch_mixed(n=4, seed0=300)
    assert b2.autotune(cache_path=str(path)) == t  # taken from the cache, not timed again
    assert (b2.mode, (b2.tuning.ctas_per_sm, b2.tuning.samples_per_thread)) == (cached['mode'],
                                                                                  tuple(cached['tuning']))
