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
