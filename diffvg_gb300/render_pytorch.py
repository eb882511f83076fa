"""PyTorch front end of the GB300 render path: pydiffvg's RenderFunction.

Drop-in for pydiffvg.RenderFunction (reference: pydiffvg/render_pytorch.py):
``serialize_scene`` builds the same flat argument list, ``apply`` takes
``(width, height, num_samples_x, num_samples_y, seed, background_image,
*args)`` and returns the ``[H, W, 4]`` image (or the ``[H, W, 1]`` /
``[N, 1]`` signed distance), autograd delivers a gradient to every argument
tensor that requires grad (the reference's backward returns None for the
non-differentiable ones) and ``render_grad`` returns the ``[H, W, 2]``
translation gradient image.

Differences from the reference that a caller can observe:
  * tensors keep their device: serialize_scene does not copy them to the
    host, and gradients come back on the device of each input tensor;
  * the scene topology (shape kinds, segment counts, group membership) is
    uploaded once and cached on the device by its hash, so an optimisation
    loop re-sends only the parameter values (one concatenated fp32 arena);
  * there is no CPU path: rendering requires a CUDA device.
"""
from collections import OrderedDict
from enum import IntEnum
import itertools
import operator
import threading
import warnings
import weakref

import torch

from . import device as _device
from . import _native
from .diffvg import ShapeType, ColorType, FilterType
from .packing import pack_scene, pack_scene_cached
from .pixel_filter import PixelFilter
from . import shape as _shape
from . import color as _color

print_timing = False


def set_print_timing(val):
    global print_timing
    print_timing = val


_fragment_cache = True


def set_fragment_cache(enabled):
    """Whether a forward render keeps each sample's fragment list on the
    device for the backward of the same parameters (no reference
    counterpart).  Off, the backward recomputes the lists as the reference
    does (diffvg.cpp:605-705): the same gradients, less device memory (about
    110 B per sample, 1.1 KB with prefiltering), a slower backward."""
    global _fragment_cache
    _fragment_cache = bool(enabled)


def get_fragment_cache():
    return _fragment_cache


class OutputType(IntEnum):
    color = 1
    sdf = 2


_SCENE_CACHE_SIZE = 64
# shared defaults, so that repeated serialize_scene calls produce the same
# argument objects (the packed-scene cache keys on tensor identity)
_EMPTY_EVAL = torch.tensor([])
_DEFAULT_FILTER = PixelFilter(type=FilterType.box, radius=torch.tensor(0.5))
_THICKNESS_PLACEHOLDER = torch.tensor(0.0)
_cache_lock = threading.Lock()
_scene_cache = OrderedDict()
_token = itertools.count(1)
_ints = {}


def _intern(v):
    """One object per integer value, so that repeated serialize_scene calls
    give argument lists of identical objects (the packing cache's identity
    key)."""
    return _ints.setdefault(v, v) if type(v) is int and len(_ints) < 4096 else v


def _native_scene(packed, device):
    """Resident device scene for this topology (cached, LRU)."""
    key = (packed.topology_key, device.index)
    with _cache_lock:
        sc = _scene_cache.get(key)
        if sc is not None:
            _scene_cache.move_to_end(key)
            return sc
    with torch.cuda.device(device):
        sc = _native.NativeScene(packed)
    sc.last_token = None
    with _cache_lock:
        _scene_cache[key] = sc
        while len(_scene_cache) > _SCENE_CACHE_SIZE:
            _, old = _scene_cache.popitem(last=False)
            old.close()
    return sc


def clear_scene_cache():
    with _cache_lock:
        for sc in _scene_cache.values():
            sc.close()
        _scene_cache.clear()


def _render_device():
    dev = _device.get_device()
    if dev.type != 'cuda':
        raise RuntimeError('diffvg_gb300 renders on CUDA only; set_use_gpu(False) has no CPU path here')
    if not torch.cuda.is_available():
        raise RuntimeError('diffvg_gb300 needs a CUDA device')
    if dev.index is None:
        dev = torch.device('cuda', torch.cuda.current_device())
    return dev


def _background(background_image, height, width, device, strict=True):
    if background_image is None:
        return None
    bg = background_image.to(device=device, dtype=torch.float32)
    if bg.shape[2] == 3:
        if strict:
            raise NotImplementedError('Background image must have 4 channels, not 3. Add a fourth channel with '
                                      'all ones via torch.ones().')
        bg = torch.cat((bg, torch.ones(bg.shape[0], bg.shape[1], 1, device=device)), dim=2)
    bg = bg.contiguous()
    assert bg.shape[0] == height and bg.shape[1] == width and bg.shape[2] == 4
    return bg


def _dims(packed, width, height, nsx, nsy):
    """The dims argument of the torch.ops.diffvg_gb300 render operators."""
    return [int(width), int(height), int(nsx), int(nsy), 1 if packed.use_prefiltering else 0]


def _eval_positions(packed, device):
    ev = packed.eval_positions
    if ev is None or ev.numel() == 0:
        return None
    return ev.to(device=device, dtype=torch.float32).reshape(-1, 2).contiguous()


class RenderFunction(torch.autograd.Function):
    """The PyTorch interface of the renderer (render_pytorch.py:18-868): a
    torch.autograd.Function with the reference's static forward(ctx, width,
    height, num_samples_x, num_samples_y, seed, background_image, *args) and
    backward(ctx, grad_img) (one gradient or None per input, in input
    order), so code that calls them directly works.  ``apply`` does not go
    through them: it hands autograd only the argument tensors that require
    grad (_RenderCore), so a step over thousands of shapes pays no
    per-argument bookkeeping for the others; the values are the same.
    """

    @staticmethod
    def serialize_scene(canvas_width, canvas_height, shapes, shape_groups,
                        filter=None, output_type=OutputType.color, use_prefiltering=False,
                        eval_positions=None):
        """Flattens a scene into RenderFunction.apply's argument list, in the
        reference's order (render_pytorch.py:22-172)."""
        if filter is None:
            filter = _DEFAULT_FILTER
        if eval_positions is None:
            eval_positions = _EMPTY_EVAL
        args = [_intern(canvas_width), _intern(canvas_height), _intern(len(shapes)), _intern(len(shape_groups)),
                output_type, use_prefiltering, eval_positions]
        for shp in shapes:
            use_thickness = False
            if isinstance(shp, _shape.Circle) or type(shp).__name__ == 'Circle':
                args += [ShapeType.circle, shp.radius, shp.center]
            elif isinstance(shp, _shape.Ellipse) or type(shp).__name__ == 'Ellipse':
                args += [ShapeType.ellipse, shp.radius, shp.center]
            elif isinstance(shp, _shape.Path) or type(shp).__name__ == 'Path':
                assert shp.points.shape[1] == 2
                args += [ShapeType.path, shp.num_control_points.to(torch.int32), shp.points]
                sw = shp.stroke_width
                if len(sw.shape) > 0 and sw.shape[0] > 1:
                    use_thickness = True
                    args.append(sw)
                else:
                    args.append(None)
                args += [shp.is_closed, getattr(shp, 'use_distance_approx', False)]
            elif isinstance(shp, _shape.Polygon) or type(shp).__name__ == 'Polygon':
                assert shp.points.shape[1] == 2
                n = shp.points.shape[0] if shp.is_closed else shp.points.shape[0] - 1
                args += [ShapeType.path, torch.zeros(n, dtype=torch.int32), shp.points, None, shp.is_closed, False]
            elif isinstance(shp, _shape.Rect) or type(shp).__name__ == 'Rect':
                args += [ShapeType.rect, shp.p_min, shp.p_max]
            else:
                raise TypeError('unknown shape type %r' % type(shp))
            args.append(_THICKNESS_PLACEHOLDER if use_thickness else shp.stroke_width)
        for grp in shape_groups:
            args.append(grp.shape_ids)
            for paint in (grp.fill_color, grp.stroke_color):
                if paint is None:
                    args.append(None)
                elif isinstance(paint, torch.Tensor):
                    args += [ColorType.constant, paint]
                elif hasattr(paint, 'begin'):
                    args += [ColorType.linear_gradient, paint.begin, paint.end, paint.offsets, paint.stop_colors]
                elif hasattr(paint, 'center'):
                    args += [ColorType.radial_gradient, paint.center, paint.radius, paint.offsets, paint.stop_colors]
                else:
                    raise TypeError('unknown paint type %r' % type(paint))
                if paint is grp.fill_color and paint is not None:
                    for sid in grp.shape_ids.tolist():
                        s = shapes[sid]
                        if type(s).__name__ == 'Path' and not s.is_closed:
                            warnings.warn('Detected non-closed paths with fill color. This might causes '
                                          'unexpected results.', Warning)
            args.append(grp.use_even_odd_rule)
            args.append(grp.shape_to_canvas.contiguous())
        args.append(filter.type)
        args.append(filter.radius)
        return args

    @staticmethod
    def apply(width, height, num_samples_x, num_samples_y, seed, background_image, *args):
        """Renders the serialized scene; differentiable with respect to every
        tensor of ``args`` (and ``background_image``) that requires grad.
        Autograd sees only those tensors, so a step over thousands of shapes
        does not pay per-argument bookkeeping for the rest of the list."""
        packed = pack_scene_cached(args)
        dims = (width, height, num_samples_x, num_samples_y, seed)
        base = _fused_base(packed)
        if base is not None:
            # a scene of fuse_parameters views: render from, and differentiate
            # with respect to, the one tensor they alias
            return _RenderCore.apply(_RenderCall(dims, packed, None, base), background_image, base)
        T = torch.Tensor
        grad_slots = [k for k, (sl, t) in enumerate(zip(packed.slots, packed.tensors))
                      if sl.differentiable and isinstance(t, T) and t.requires_grad]
        call = _RenderCall(dims, packed, grad_slots)
        return _RenderCore.apply(call, background_image, *[packed.tensors[k] for k in grad_slots])

    @staticmethod
    def forward(ctx, width, height, num_samples_x, num_samples_y, seed, background_image, *args):
        """The render (render_pytorch.py:174-428); keeps on ctx what
        backward needs, for every differentiable argument."""
        packed = pack_scene_cached(args)
        slots = [k for k, sl in enumerate(packed.slots) if sl.differentiable]
        call = _RenderCall((width, height, num_samples_x, num_samples_y, seed), packed, slots)
        ctx.num_args = len(args)
        return _render_forward(ctx, call, background_image)

    @staticmethod
    def backward(ctx, grad_img):
        """Gradients of <grad_img, render> for every input of forward, in
        input order (render_pytorch.py:668-868): None for the image size,
        sample counts, seed and the non-differentiable arguments; the
        background gradient when a background was given."""
        d_bg, grads = _render_backward(ctx, grad_img)
        out = [None] * ctx.num_args
        for k, g in zip(ctx.grad_slots, grads):
            out[ctx.packed.slots[k].arg_index] = g
        return (None, None, None, None, None, d_bg) + tuple(out)

    @staticmethod
    def render_grad(grad_img, width, height, num_samples_x, num_samples_y, seed, background_image, *args):
        """Gradient of <grad_img, render> with respect to a screen-space
        translation of every pixel's content: a [H, W, 2] image
        (render_pytorch.py:430-666)."""
        device = _render_device()
        packed = pack_scene(args)
        scene = _native_scene(packed, device)
        arena = packed.param_arena(device).contiguous()
        ev = _eval_positions(packed, device)
        grad = grad_img.to(device=device, dtype=torch.float32).contiguous()
        if packed.output_type == OutputType.color:
            assert grad.shape[2] == 4
        else:
            assert grad.shape[2] == 1
        bg = _background(background_image, height, width, device, strict=False)
        d_translation = torch.zeros(height, width, 2, device=device)
        d_arena = torch.zeros(max(packed.num_params, 1), device=device)
        dims = _dims(packed, width, height, num_samples_x, num_samples_y)
        color = packed.output_type == OutputType.color
        with torch.cuda.device(device):
            scene.render_backward(dims, seed, d_arena, params=arena, background=bg, eval_positions=ev,
                                  d_image=grad if color else None, d_sdf=None if color else grad,
                                  d_translation=d_translation)
        scene.last_token = None
        return d_translation


class _RenderCall:
    """What one RenderFunction.apply call renders: image size, sample
    counts, seed, the packed scene and the slots whose tensors autograd
    tracks, or the fused parameter tensor (fuse_parameters) it renders from
    and differentiates with respect to."""
    __slots__ = ('dims', 'packed', 'grad_slots', 'fused')

    def __init__(self, dims, packed, grad_slots, fused=None):
        self.dims, self.packed, self.grad_slots, self.fused = dims, packed, grad_slots, fused


# fuse_parameters tensors by storage address
_fused = weakref.WeakValueDictionary()


def fuse_parameters(canvas_width, canvas_height, shapes, shape_groups, filter=None):
    """One parameter tensor for a whole scene (no reference counterpart).

    Gathers every parameter tensor that serialize_scene passes for these
    objects (radii, centres, points, thicknesses, stroke widths, corners,
    paints and their stops, group transforms, the filter radius) into one
    fp32 leaf tensor on the render device, in the renderer's parameter
    layout, and rebinds each object's attribute to a view of it (a detached
    alias: the objects read the current values, autograd does not track
    them).  RenderFunction.apply on a scene serialized from these objects
    then renders straight from that tensor and hands autograd that one
    tensor: its .grad receives the whole gradient in one piece, where
    separate leaf tensors cost autograd one node each.  Optimise it as one
    parameter (``torch.optim.Adam([arena])``); the objects see the updates
    through their views.  A tensor that several attributes share (such as
    ShapeGroup's default transform) becomes one view per attribute, i.e.
    separate parameters.  Returns (arena, filter): pass the filter to
    serialize_scene (a new box filter of radius 0.5 when none is given, so
    that its radius is in the tensor too).  A scene whose arguments are not
    exactly these views (an attribute replaced later) renders through the
    per-tensor path."""
    if filter is None:
        filter = PixelFilter(type=FilterType.box, radius=torch.tensor(0.5))
    shape_names = ('radius', 'center', 'points', 'stroke_width', 'p_min', 'p_max')
    paint_names = ('begin', 'end', 'center', 'radius', 'offsets', 'stop_colors')
    owners = [(shp, shape_names) for shp in shapes]
    for grp in shape_groups:
        owners.append((grp, ('fill_color', 'stroke_color', 'shape_to_canvas')))
        for paint in (grp.fill_color, grp.stroke_color):
            if paint is not None and not isinstance(paint, torch.Tensor):
                owners.append((paint, paint_names))
    owners.append((filter, ('radius',)))
    seen = set()
    for obj, names in owners:  # one tensor object per attribute
        for nm in names:
            t = getattr(obj, nm, None)
            if isinstance(t, torch.Tensor):
                if id(t) in seen:
                    setattr(obj, nm, t.detach().clone())
                else:
                    seen.add(id(t))
    args = RenderFunction.serialize_scene(canvas_width, canvas_height, shapes, shape_groups, filter=filter)
    packed = pack_scene(args)
    device = _render_device()
    with torch.no_grad():
        arena = packed.param_arena(device).detach().clone().contiguous()
    arena.requires_grad_(True)
    data = arena.detach()
    views = {}
    for sl, t in zip(packed.slots, packed.tensors):
        if isinstance(t, torch.Tensor) and id(t) not in views:
            views[id(t)] = data[sl.offset:sl.offset + sl.numel].view(sl.shape)

    for obj, names in owners:
        for nm in names:
            t = getattr(obj, nm, None)
            if isinstance(t, torch.Tensor) and id(t) in views:
                setattr(obj, nm, views[id(t)])
    _fused[data.untyped_storage().data_ptr()] = arena
    return arena, filter


def _fused_base(packed):
    """The fuse_parameters tensor that every parameter slot of packed is a
    view of, at the slot's offset, or None.  Decided once per packed scene
    (the packing cache returns the same object for the same arguments)."""
    hit = getattr(packed, '_fused_base', False)
    if hit is not False:
        base = hit() if hit is not None else None
        return base
    base = None
    ts = packed.tensors
    if ts and isinstance(ts[0], torch.Tensor) and ts[0].is_cuda:
        cand = _fused.get(ts[0].untyped_storage().data_ptr())
        if cand is not None and cand.numel() == packed.num_params:
            ptr, off0 = cand.untyped_storage().data_ptr(), cand.storage_offset()
            ok = True
            for sl, t in zip(packed.slots, ts):
                if not (isinstance(t, torch.Tensor) and t.dtype == torch.float32 and t.is_contiguous() and
                        t.untyped_storage().data_ptr() == ptr and t.storage_offset() == off0 + sl.offset):
                    ok = False
                    break
            if ok:
                base = cand
    packed._fused_base = weakref.ref(base) if base is not None else None
    return base


def _render_forward(ctx, call, background_image):
    """Forward render of `call` into a new output tensor; keeps on ctx what
    _render_backward needs (render_pytorch.py:186-428)."""
    width, height, num_samples_x, num_samples_y, seed = call.dims
    packed = call.packed
    device = _render_device()
    scene = _native_scene(packed, device)
    fused = call.fused if call.fused is not None and call.fused.device == device else None
    arena = fused.detach() if fused is not None else packed.param_arena(device).contiguous()
    ev = _eval_positions(packed, device)
    if packed.output_type == OutputType.color:
        assert ev is None, 'eval_positions apply to the sdf output only'
        out = torch.empty(height, width, 4, device=device)
    else:
        out = torch.empty((height, width, 1) if ev is None else (ev.shape[0], 1), device=device)
    bg = _background(background_image, out.shape[0], out.shape[1], device)
    if not bool(torch.isfinite(arena).all()):
        raise ValueError('scene parameters contain a non-finite value')
    token = next(_token)
    flags = 0 if _fragment_cache else _native.DVG_FLAG_NO_FRAG_CACHE
    dims = _dims(packed, width, height, num_samples_x, num_samples_y)
    color = packed.output_type == OutputType.color
    with torch.cuda.device(device):
        scene.render_forward(dims, seed, flags, params=arena, background=bg, eval_positions=ev,
                             image=out if color else None, sdf=None if color else out)
    scene.last_token = token
    ctx.packed = packed
    ctx.scene = scene
    ctx.arena = arena
    ctx.token = token
    ctx.background_image = bg
    ctx.bg_requested = background_image is not None
    ctx.eval_positions = ev
    ctx.dims = call.dims
    ctx.device = device
    ctx.grad_slots = call.grad_slots
    ctx.fused = call.fused
    ctx.fused_version = call.fused._version if call.fused is not None else None
    return out


_device_of = operator.attrgetter('device')
_dtype_of = operator.attrgetter('dtype')


def _render_backward(ctx, grad_img):
    """The backward render of a _render_forward (render_pytorch.py:668-868):
    (background gradient or None, gradients of the call's slots in
    ctx.grad_slots order, each on its input's device)."""
    packed, scene, device = ctx.packed, ctx.scene, ctx.device
    width, height, nsx, nsy, seed = ctx.dims
    fused = getattr(ctx, 'fused', None)
    if fused is not None and fused._version != ctx.fused_version:
        raise RuntimeError('the fused parameter tensor was modified in place between the render and its backward')
    grad = grad_img.to(device=device, dtype=torch.float32).contiguous()
    d_arena = torch.zeros(max(packed.num_params, 1), device=device)
    bg = ctx.background_image
    d_bg = torch.zeros_like(bg) if bg is not None else None
    reuse = _native.DVG_FLAG_REUSE_PREP if scene.last_token == ctx.token else 0
    stream = torch.cuda.current_stream(device).cuda_stream

    dims = _dims(packed, width, height, nsx, nsy)
    color = packed.output_type == OutputType.color

    def launch(flags):
        with torch.cuda.device(device):
            scene.render_backward(dims, seed, d_arena, flags, params=ctx.arena, background=bg,
                                  eval_positions=ctx.eval_positions, d_image=grad if color else None,
                                  d_sdf=None if color else grad, d_background=d_bg if color else None)

    # the kernels run while the host lays out the gradient views; the
    # status is checked once the gradient has been read back
    launch(reuse | _native.DVG_FLAG_NO_SYNC)
    scene.last_token = ctx.token
    tensors = packed.tensors
    if fused is not None:
        # one gradient: the fused tensor's, the arena itself
        bufs = {device: d_arena}
        if fused.device != device:
            bufs[fused.device] = torch.empty(d_arena.shape, dtype=torch.float32, device=fused.device)
        grads = [bufs[fused.device][:fused.numel()]]
    else:
        # one view of the gradient arena per slot, on its tensor's device and
        # in its dtype (arena_views builds the views in one call)
        ts = [tensors[k] for k in ctx.grad_slots]
        dsts = set(map(_device_of, ts))
        bufs = {device: d_arena}
        for dst in dsts:
            if dst != device:
                bufs[dst] = torch.empty(d_arena.shape, dtype=torch.float32, device=dst)
        spec = packed.grad_view_spec(ctx.grad_slots)
        views = {dst: _native.ops().arena_views(bufs[dst], *spec) for dst in dsts}
        if len(views) <= 1:
            grads = list(views.popitem()[1]) if views else []
        else:
            grads = [views[t.device][i] for i, t in enumerate(ts)]
        if ts and set(map(_dtype_of, ts)) != {torch.float32}:
            grads = [g if t.dtype == g.dtype else g.to(t.dtype) for g, t in zip(grads, ts)]
    for dst, b in bufs.items():
        if dst != device:
            b.copy_(d_arena)  # waits for the kernels
    try:
        scene.sync(stream)
    except _native.SceneCapacityError as e:
        if 'grown' not in str(e):
            raise
        # the tile lists outgrew their capacity and were grown: the
        # gradient is computed again, synchronously
        d_arena.zero_()
        if d_bg is not None:
            d_bg.zero_()
        launch(0)
        for dst, b in bufs.items():
            if dst != device:
                b.copy_(d_arena)
    return (d_bg if ctx.bg_requested else None), grads


class _RenderCore(torch.autograd.Function):
    """Forward and backward of one render: inputs are the tensors that
    require grad, in slot order."""

    @staticmethod
    def forward(ctx, call, background_image, *grad_tensors):
        return _render_forward(ctx, call, background_image)

    @staticmethod
    def backward(ctx, grad_img):
        d_bg, grads = _render_backward(ctx, grad_img)
        return (None, d_bg) + tuple(grads)
