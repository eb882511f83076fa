"""Host-side packing: the packed-scene cache of optimisation loops and the
parameter arena (CPU only)."""
import torch

import diffvg_gb300 as dvg
from diffvg_gb300 import workloads
from diffvg_gb300.packing import pack_scene, pack_scene_cached


def _scene():
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=7, num_paths=6, canvas=64)
    return w, h, shapes, groups


def test_cache_hits_for_the_same_objects():
    w, h, shapes, groups = _scene()
    a = pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    b = pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    assert a is b


def test_cache_misses_after_an_inplace_topology_edit():
    w, h, shapes, groups = _scene()
    a = pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    shapes[0].num_control_points[0] = 1  # cubic -> quadratic: a different topology, same tensor object
    shapes[0].points = shapes[0].points[:-1].clone()
    b = pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    assert a is not b
    assert b.topology_key != a.topology_key


def test_cache_misses_after_a_resize_and_for_other_values():
    w, h, shapes, groups = _scene()
    a = pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    c = pack_scene_cached(dvg.RenderFunction.serialize_scene(w + 1, h, shapes, groups))
    assert c is not a and c.canvas_width == w + 1
    pts = shapes[1].points
    with torch.no_grad():
        pts.resize_(pts.shape[0], 2)  # same shape: still a hit
    assert pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups)) is a
    shapes[1].stroke_width.resize_(1)  # 0-d -> 1-d in place: a miss
    d = pack_scene_cached(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    assert d is not a


def test_param_arena_is_the_slots_in_order():
    w, h, shapes, groups = _scene()
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    arena = packed.param_arena(torch.device('cpu'))
    assert arena.numel() == packed.num_params
    for sl, t in zip(packed.slots, packed.tensors):
        got = arena[sl.offset:sl.offset + sl.numel]
        assert torch.equal(got, t.detach().reshape(-1).to(torch.float32))
