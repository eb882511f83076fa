"""torch.ops.diffvg_gb300 on the GPU: a direct operator call renders what
RenderFunction renders, and tensors of the wrong size or device are refused
before the render runs."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _scene():
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads, _native
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=3, num_paths=12, canvas=64)
    args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
    packed = pack_scene(args)
    dev = torch.device('cuda', 0)
    with torch.cuda.device(dev):
        scene = _native.NativeScene(packed)
    return dvg, args, packed, scene, w, h, dev


def test_operator_render_matches_render_function():
    dvg, args, packed, scene, w, h, dev = _scene()
    from diffvg_gb300 import _native
    ops = _native.ops()
    arena = packed.param_arena(dev).contiguous()
    img = torch.empty(h, w, 4, device=dev)
    _native.check(ops.render_forward(scene.handle.value, arena, None, None, img, None, [w, h, 2, 2, 0], 5, 0))
    ref = dvg.RenderFunction.apply(w, h, 2, 2, 5, None, *args)
    assert torch.equal(img, ref)
    d_params = torch.zeros(packed.num_params, device=dev)
    _native.check(ops.render_backward(scene.handle.value, arena, None, None, torch.ones_like(img), None, d_params,
                                      None, None, [w, h, 2, 2, 0], 5, 0))
    assert bool(torch.isfinite(d_params).all()) and float(d_params.abs().sum()) > 0
    scene.close()


def test_operator_refuses_short_or_misplaced_tensors():
    dvg, args, packed, scene, w, h, dev = _scene()
    from diffvg_gb300 import _native
    ops = _native.ops()
    h_ = scene.handle.value
    arena = packed.param_arena(dev).contiguous()
    img = torch.empty(h, w, 4, device=dev)
    dims = [w, h, 2, 2, 0]
    with pytest.raises(RuntimeError, match='params has'):
        ops.render_forward(h_, arena[:-1], None, None, img, None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='image has'):
        ops.render_forward(h_, arena, None, None, img[:-1], None, dims, 0, 0)
    with pytest.raises(RuntimeError, match="scene's device"):
        ops.render_forward(h_, arena, None, None, torch.empty(h, w, 4), None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='d_params has'):
        ops.render_backward(h_, arena, None, None, torch.ones_like(img), None, torch.zeros(packed.num_params - 1,
                            device=dev), None, None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='params has'):
        ops.scene_update_params(h_, arena[:-1])
    scene.close()
