"""RenderFunction.apply through autograd: gradients reach exactly the
argument tensors that require grad, with the same values whichever subset
requires it."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _scene(dvg):
    from diffvg_gb300 import workloads
    return workloads.stroke_scene(dvg, seed=11, num_paths=24, canvas=96)


def _grads(requires):
    import diffvg_gb300 as dvg
    w, h, shapes, groups = _scene(dvg)
    for s in shapes:
        s.points.requires_grad_('points' in requires)
        s.stroke_width.requires_grad_('width' in requires)
    for g in groups:
        g.stroke_color.requires_grad_('color' in requires)
    args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
    img = dvg.RenderFunction.apply(w, h, 2, 2, 3, None, *args)
    loss = (img * torch.linspace(0, 1, img.numel(), device=img.device).reshape(img.shape)).sum()
    loss.backward()
    return shapes, groups


def test_gradients_follow_requires_grad():
    s_all, g_all = _grads({'points', 'width', 'color'})
    s_pts, g_pts = _grads({'points'})
    for a, b in zip(s_all, s_pts):
        assert b.points.grad is not None and b.stroke_width.grad is None
        torch.testing.assert_close(b.points.grad, a.points.grad, rtol=1e-4, atol=1e-5)
    for a, b in zip(g_all, g_pts):
        assert b.stroke_color.grad is None and a.stroke_color.grad is not None


def test_no_grad_render_needs_no_autograd():
    import diffvg_gb300 as dvg
    w, h, shapes, groups = _scene(dvg)
    with torch.no_grad():
        img = dvg.RenderFunction.apply(w, h, 2, 2, 3, None, *dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    assert img.shape == (h, w, 4) and not img.requires_grad


def test_direct_forward_backward_like_the_reference():
    """RenderFunction is a torch.autograd.Function whose static forward /
    backward can be called directly (render_pytorch.py:174, 668): backward
    returns one entry per forward input, the gradients at the differentiable
    arguments' positions equal what autograd delivers through apply, None
    elsewhere."""
    import diffvg_gb300 as dvg
    assert issubclass(dvg.RenderFunction, torch.autograd.Function)
    shapes, groups = _grads({'points', 'width', 'color'})
    w, h, shapes2, groups2 = _scene(dvg)
    args = dvg.RenderFunction.serialize_scene(w, h, shapes2, groups2)

    class Ctx:
        pass
    ctx = Ctx()
    img = dvg.RenderFunction.forward(ctx, w, h, 2, 2, 3, None, *args)
    grad = torch.linspace(0, 1, img.numel(), device=img.device).reshape(img.shape)
    out = dvg.RenderFunction.backward(ctx, grad)
    assert len(out) == 6 + len(args)
    assert all(x is None for x in out[:6])
    for pos, a in enumerate(args):
        g = out[6 + pos]
        if g is not None:
            assert isinstance(a, torch.Tensor) and g.shape == a.shape
    idx = {id(a): 6 + k for k, a in enumerate(args)}
    for a, b in zip(shapes, shapes2):
        torch.testing.assert_close(out[idx[id(b.points)]], a.points.grad, rtol=1e-4, atol=1e-5)
        torch.testing.assert_close(out[idx[id(b.stroke_width)]], a.stroke_width.grad, rtol=1e-4, atol=1e-5)
    for a, b in zip(groups, groups2):
        torch.testing.assert_close(out[idx[id(b.stroke_color)]], a.stroke_color.grad, rtol=1e-4, atol=1e-5)
        assert out[idx[id(b.shape_ids)]] is None


def test_fused_parameters_give_the_per_tensor_gradients():
    """fuse_parameters: the scene renders from one leaf tensor whose .grad
    holds, at each attribute's place, the gradient the per-tensor path
    delivers to that attribute; an Adam step on it moves the objects."""
    import diffvg_gb300 as dvg
    from diffvg_gb300.render_pytorch import _fused_base
    from diffvg_gb300.packing import pack_scene_cached
    shapes, groups = _grads({'points', 'width', 'color'})
    w, h, shapes2, groups2 = _scene(dvg)
    arena, filt = dvg.fuse_parameters(w, h, shapes2, groups2)
    assert arena.is_leaf and arena.requires_grad and arena.is_cuda
    args = dvg.RenderFunction.serialize_scene(w, h, shapes2, groups2, filter=filt)
    assert _fused_base(pack_scene_cached(args)) is arena
    img = dvg.RenderFunction.apply(w, h, 2, 2, 3, None, *args)
    loss = (img * torch.linspace(0, 1, img.numel(), device=img.device).reshape(img.shape)).sum()
    loss.backward()
    data = arena.detach()
    for a, b in zip(shapes, shapes2):
        off = (b.points.storage_offset() - data.storage_offset())
        g = arena.grad[off:off + b.points.numel()].view(b.points.shape)
        torch.testing.assert_close(g, a.points.grad.to(g.device), rtol=1e-4, atol=1e-5)
        off = (b.stroke_width.storage_offset() - data.storage_offset())
        torch.testing.assert_close(arena.grad[off].reshape(a.stroke_width.grad.shape),
                                   a.stroke_width.grad.to(arena.device), rtol=1e-4, atol=1e-5)
    for a, b in zip(groups, groups2):
        off = (b.stroke_color.storage_offset() - data.storage_offset())
        torch.testing.assert_close(arena.grad[off:off + 4], a.stroke_color.grad.to(arena.device), rtol=1e-4,
                                   atol=1e-5)
    before = shapes2[0].points.clone()
    opt = torch.optim.Adam([arena], lr=0.5)
    opt.step()
    assert not torch.equal(before, shapes2[0].points)
    # a replaced attribute leaves the fused path: the per-tensor path renders the same image
    shapes2[0].points = shapes2[0].points.clone()
    args = dvg.RenderFunction.serialize_scene(w, h, shapes2, groups2, filter=filt)
    assert _fused_base(pack_scene_cached(args)) is None
    img2 = dvg.RenderFunction.apply(w, h, 2, 2, 3, None, *args)
    args3 = dvg.RenderFunction.serialize_scene(w, h, shapes2, groups2, filter=filt)
    torch.testing.assert_close(img2, dvg.RenderFunction.apply(w, h, 2, 2, 3, None, *args3))


@pytest.mark.parametrize('prefilter', [False, True])
def test_fragment_cache_off_gives_the_same_render_and_gradients(prefilter):
    """With set_fragment_cache(False) the forward keeps no fragment lists and
    the backward recomputes them: the image is bit-identical and the
    gradients equal the cached path's up to the order of the atomic sums
    (relative 1e-4 of the largest gradient entry)."""
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads

    def run(cache):
        if prefilter:
            w, h, shapes, groups = workloads.fill_scene(dvg, seed=9, num_paths=64, canvas=96)
        else:
            w, h, shapes, groups = workloads.mixed_scene(dvg, 77, 96, 400)
        leaves = []
        for s in shapes:
            s.points.requires_grad_(True)
            leaves.append(s.points)
        for g in groups:
            for attr in ('fill_color', 'stroke_color'):
                c = getattr(g, attr)
                if isinstance(c, torch.Tensor):
                    c.requires_grad_(True)
                    leaves.append(c)
        dvg.set_fragment_cache(cache)
        try:
            args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=prefilter)
            img = dvg.RenderFunction.apply(w, h, 1 if prefilter else 2, 1 if prefilter else 2, 5, None, *args)
            (img * torch.linspace(0, 1, img.numel(), device=img.device).reshape(img.shape)).sum().backward()
        finally:
            dvg.set_fragment_cache(True)
        return img.detach(), torch.cat([t.grad.reshape(-1).cpu() for t in leaves])

    img_on, g_on = run(True)
    img_off, g_off = run(False)
    assert torch.equal(img_on, img_off)
    scale = float(g_on.abs().max())
    assert scale > 0
    assert float((g_on - g_off).abs().max()) <= 1e-4 * scale
