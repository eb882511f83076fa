"""The PyTorch operators over the C ABI (torch.ops.diffvg_gb300,
diffvg_gb300/csrc/dvg_torch.cpp): registration, host-side argument checks
and status codes, all without a GPU."""
import pytest
import torch

from diffvg_gb300 import _native

OPS = {
    'scene_create': 'scene_create(Tensor shape_info, Tensor segment_ctrl, Tensor group_info, Tensor group_shapes, '
                    'int[] dims) -> (int, int)',
    'scene_destroy': 'scene_destroy(int scene) -> int',
    'render_forward': 'render_forward(int scene, Tensor? params, Tensor? background, Tensor? eval_positions, '
                      'Tensor(a!)? image, Tensor(b!)? sdf, int[] dims, int seed, int flags) -> int',
    'render_backward': 'render_backward(int scene, Tensor? params, Tensor? background, Tensor? eval_positions, '
                       'Tensor? d_image, Tensor? d_sdf, Tensor(a!) d_params, Tensor(b!)? d_background, '
                       'Tensor(c!)? d_translation, int[] dims, int seed, int flags) -> int',
    'scene_update_params': 'scene_update_params(int scene, Tensor params) -> int',
    'scene_sync': 'scene_sync(int scene, int device) -> int',
    'arena_views': 'arena_views(Tensor(a -> *) arena, int[] offsets, int[] numels, int[] ndims, int[] dims) '
                   '-> Tensor(a)[]',
}


def test_operators_are_registered_with_their_schemas():
    ops = _native.ops()
    for name, schema in OPS.items():
        assert str(getattr(ops, name).default._schema) == 'diffvg_gb300::' + schema


def test_scene_create_reports_a_malformed_description_without_touching_the_device():
    ops = _native.ops()
    z = torch.zeros(1, dtype=torch.int32)
    st, handle = ops.scene_create(z, z[:0], z, z[:0], [0, 16, 0, 0, 1, 0, 0])  # canvas width 0
    assert st == _native.DVG_ERR_INVALID and handle == 0
    assert b'canvas' in _native.load().dvg_last_error()


def test_scene_create_takes_int32_cpu_topology_only():
    ops = _native.ops()
    z = torch.zeros(1, dtype=torch.int64)
    with pytest.raises(RuntimeError, match='int32 CPU'):
        ops.scene_create(z, z, z, z, [16, 16, 0, 0, 1, 0, 0])


def test_render_operators_check_arguments_before_the_call():
    """Malformed arguments fail in the operator before any render entry point
    runs: the dims list, the output choice, and the scene handle (a NULL
    handle is reported by dvg_scene_info; tensors are then checked against
    the scene's parameter count and device)."""
    ops = _native.ops()
    dims = [8, 8, 1, 1, 0]
    cpu = torch.zeros(8, 8, 4)
    with pytest.raises(RuntimeError, match='dims'):
        ops.render_forward(0, None, None, None, cpu, None, [8, 8], 0, 0)
    with pytest.raises(RuntimeError, match='exactly one of image / sdf'):
        ops.render_forward(0, None, None, None, None, None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='invalid scene handle'):
        ops.render_forward(0, None, None, None, cpu, None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='exactly one of d_image / d_sdf'):
        ops.render_backward(0, None, None, None, None, None, torch.zeros(4), None, None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='invalid scene handle'):
        ops.render_backward(0, None, None, None, cpu, None, torch.zeros(4), None, None, dims, 0, 0)
    with pytest.raises(RuntimeError, match='invalid scene handle'):
        ops.scene_update_params(0, torch.zeros(4))


def test_scene_info_reports_a_null_scene():
    import ctypes
    lib = _native.load()
    n = ctypes.c_int32(-7)
    assert lib.dvg_scene_info(None, ctypes.byref(n), None) == _native.DVG_ERR_INVALID
    assert n.value == -7


def test_seeds_keep_their_64_bits():
    assert _native._i64(0) == 0
    assert _native._i64(2 ** 63) == -2 ** 63
    assert _native._i64(2 ** 64 - 1) == -1
    assert _native._i64(-1) == -1


def test_arena_views_alias_the_arena_in_slot_shapes():
    """The gradient views RenderFunction's backward returns: each slot's
    floats of the one arena, in the slot's shape, sharing its storage."""
    ops = _native.ops()
    arena = torch.arange(20, dtype=torch.float32)
    views = ops.arena_views(arena, [0, 4, 10, 19], [4, 6, 9, 1], [1, 2, 2, 0], [4, 3, 2, 3, 3])
    assert [tuple(v.shape) for v in views] == [(4,), (3, 2), (3, 3), ()]
    assert [v.data_ptr() - arena.data_ptr() for v in views] == [0, 16, 40, 76]
    assert views[1].tolist() == [[4.0, 5.0], [6.0, 7.0], [8.0, 9.0]]
    arena[19] = -1.0
    assert float(views[3]) == -1.0
    with pytest.raises(RuntimeError, match='outside the arena'):
        ops.arena_views(arena, [15], [6], [1], [6])
    with pytest.raises(RuntimeError, match='too few entries'):
        ops.arena_views(arena, [0], [6], [2], [6])
    with pytest.raises(RuntimeError, match='differ in length'):
        ops.arena_views(arena, [0, 1], [1], [1], [1])
