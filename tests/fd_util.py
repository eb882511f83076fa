"""Finite-difference checks of the renderer's gradients, shared by the oracle
(CPU) and CUDA-path (GPU) tests.

The image of a Monte-Carlo renderer is piecewise constant in the geometry at
a fixed seed, so a raw finite difference of it is noise.  The estimators
here are therefore explicit:

- colour parameters: the image is smooth in them at a fixed seed, so one
  central difference (h = 1e-2, loss summed in float64) is compared with the
  analytic gradient at a 1e-3 relative tolerance;
- geometry through the boundary (edge-sampling) term: central differences
  with a step of a quarter pixel, with the same seed on both sides (the same
  sample positions, so the difference counts the samples the boundary
  sweeps), averaged over several seeds, against the analytic gradient
  averaged over the same seeds;
- prefiltered coverage: deterministic and smooth in the geometry, so one
  central difference per parameter.

The loss is L = sum(image * weights) with a fixed smooth weight image, whose
gradient is the backward pass with d_image = weights.
"""
import numpy as np


def weight_image(h, w):
    """Smooth per-pixel, per-channel loss weights (a ramp, so that
    translations of a shape change the loss)."""
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    ramp = 1.0 + x / w + 2.0 * y / h
    ch = np.array([1.0, 0.5, 0.25, 0.1])
    return (ramp[:, :, None] * ch[None, None, :]).astype(np.float32)


def loss(image, weights):
    return float(np.sum(image.astype(np.float64) * weights.astype(np.float64)))


def slot_offset(packed, arg_index):
    """Parameter-arena offset of the argument list entry arg_index."""
    for sl in packed.slots:
        if sl.arg_index == arg_index:
            return sl.offset
    raise KeyError(arg_index)


def central_fd(fwd, P, index, h, weights, seeds):
    """Mean over seeds of (L(P + h e_i) - L(P - h e_i)) / 2h."""
    vals = []
    for seed in seeds:
        Pp = P.copy()
        Pm = P.copy()
        Pp[index] += h
        Pm[index] -= h
        vals.append((loss(fwd(Pp, seed), weights) - loss(fwd(Pm, seed), weights)) / (2.0 * h))
    return float(np.mean(vals))


def analytic(bwd, P, weights, seeds):
    """Mean over seeds of the backward pass's gradient of L."""
    return np.mean([bwd(P, seed, weights).astype(np.float64) for seed in seeds], axis=0)


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def slot_of(packed, kind, nth=0):
    """Arena offset of the nth parameter slot of the given kind."""
    found = [sl for sl in packed.slots if sl.kind == kind]
    return found[nth].offset


def circle_case(m):
    """A filled circle inside a 48x48 canvas, 4x4 spp."""
    import torch
    shapes = [m.Circle(radius=torch.tensor(12.0), center=torch.tensor([22.0, 25.0]))]
    groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=torch.tensor([0.3, 0.6, 0.3, 1.0]))]
    return 48, 48, shapes, groups, False, 4


def prefiltered_polygon_case(m):
    """A filled pentagon (lines) under prefiltering, 1 spp at pixel centres."""
    import math
    import torch
    pts = [[24.0 + 15.0 * math.cos(0.3 + 2 * math.pi * k / 5), 24.0 + 13.0 * math.sin(0.3 + 2 * math.pi * k / 5)]
           for k in range(5)]
    shapes = [m.Polygon(points=torch.tensor(pts), is_closed=True)]
    groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=torch.tensor([0.8, 0.3, 0.2, 1.0]))]
    return 48, 48, shapes, groups, True, 1


def run_checks(make_backend):
    """Runs the three finite-difference checks through a backend factory:
    make_backend(case_builder) -> (packed, P, fwd(P, seed) -> image,
    bwd(P, seed, d_image) -> d_params).  Returns the relative errors."""
    out = {}
    # colour gradients of the circle at one seed
    packed, P, fwd, bwd = make_backend(circle_case)
    wts = weight_image(48, 48)
    co = slot_of(packed, 'color')
    g = analytic(bwd, P, wts, [1])
    fd = [central_fd(fwd, P, co + k, 1e-2, wts, [1]) for k in range(4)]
    out['color'] = rel_err(fd, g[co:co + 4])
    # radius and centre through the boundary term, averaged over seeds
    seeds = list(range(1, 9))
    ro, ce = slot_of(packed, 'radius'), slot_of(packed, 'center')
    g = analytic(bwd, P, wts, seeds)
    idx = [ro, ce, ce + 1]
    fd = [central_fd(fwd, P, i, 0.25, wts, seeds) for i in idx]
    out['geometry'] = rel_err(fd, g[idx])
    # prefiltered polygon: every vertex coordinate, deterministic.  Alpha
    # only: the output colour is un-premultiplied, so a pixel's rgb jumps from
    # 0 to the paint colour where its coverage leaves 0 (alpha is smooth).
    packed, P, fwd, bwd = make_backend(prefiltered_polygon_case)
    po = slot_of(packed, 'points')
    wa = wts.copy()
    wa[:, :, :3] = 0.0
    g = analytic(bwd, P, wa, [0])
    idx = list(range(po, po + 10))
    fd = [central_fd(fwd, P, i, 1e-2, wa, [0]) for i in idx]
    out['prefiltered_points'] = rel_err(fd, g[idx])
    return out


def stroke_case(m):
    """An open cubic path, stroked (half width 1.5), 48x48, 4x4 spp."""
    import torch
    pts = torch.tensor([[6.0, 30.0], [14.0, 6.0], [30.0, 42.0], [42.0, 14.0]])
    shapes = [m.Path(num_control_points=torch.tensor([2], dtype=torch.int32), points=pts, is_closed=False,
                     stroke_width=torch.tensor(1.5))]
    groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None,
                           stroke_color=torch.tensor([0.2, 0.5, 0.9, 1.0]))]
    return 48, 48, shapes, groups, False, 4


def gradient_case(m):
    """A rect filled with a 3-stop linear gradient, 48x48, 2x2 spp."""
    import torch
    g = m.LinearGradient(begin=torch.tensor([8.0, 10.0]), end=torch.tensor([40.0, 36.0]),
                         offsets=torch.tensor([0.0, 0.45, 1.0]),
                         stop_colors=torch.tensor([[1.0, 0.0, 0.0, 1.0], [0.0, 1.0, 0.0, 0.8], [0.0, 0.0, 1.0, 1.0]]))
    shapes = [m.Rect(p_min=torch.tensor([4.0, 6.0]), p_max=torch.tensor([44.0, 42.0]))]
    groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=g)]
    return 48, 48, shapes, groups, False, 2


def run_extra_checks(make_backend):
    """The stroke width through the boundary term (averaged over seeds) and
    linear-gradient parameters (smooth at a fixed seed).

    A stroke's control-point gradients are not compared: the reference's
    boundary term for stroke geometry leaves out the offset curves' length
    factor (see the notes above run_paint_checks), and the renderer
    reproduces the reference's estimator."""
    out = {}
    wts = weight_image(48, 48)
    packed, P, fwd, bwd = make_backend(stroke_case)
    seeds = list(range(1, 9))
    sw = slot_of(packed, 'stroke_width')
    g = analytic(bwd, P, wts, seeds)
    out['stroke_width'] = rel_err([central_fd(fwd, P, sw, 0.25, wts, seeds)], g[[sw]])
    packed, P, fwd, bwd = make_backend(gradient_case)
    gb = slot_of(packed, 'gradient_geometry')   # begin, end; then stop offsets and stop colours
    so, sc = slot_of(packed, 'stop_offsets'), slot_of(packed, 'color')
    idx = list(range(gb, gb + 4)) + list(range(so, so + 3)) + list(range(sc, sc + 12))
    g = analytic(bwd, P, wts, [3])
    fd = [central_fd(fwd, P, i, 1e-2, wts, [3]) for i in idx]
    out['linear_gradient'] = rel_err(fd, g[idx])
    return out


# ---------------------------------------------------------------------------
# Every paint kind on fills and on strokes.  The reference renders gradient
# strokes wrongly and crashes in their backward pass (scene.cpp:866-869
# stores the d_color buffer over the stroke colour), so for gradient-coloured
# strokes finite differences are the only check.
#
# What finite differences can hold the reference's estimator to, and what
# not (this project reproduces the estimator, so the same holds here):
# - paint parameters (interior term): exact, except that the radial
#   gradient's adjoint also adds d_color to its last stop for every sample
#   (diffvg.cpp:441-499 has no return after the matching stop), so the last
#   stop's colour is left out for radial paints;
# - a stroke's width (boundary term): exact;
# - a stroke's geometry (points, centre, radius, group transform) through the
#   boundary term: biased.  The boundary samples sit at +-r along the centre
#   line's normal with the centre line's length density, without the offset
#   curve's length factor (1 +- r * curvature); a circle stroke's centre
#   gradient comes out at half its finite difference, for instance, and its
#   radius gradient adds the inner edge with the outer edge's sign
#   (diffvg.cpp:149-156).  Not compared.
# - path points under a non-identity group transform: the boundary term
#   takes the points' velocity in shape space as canvas velocity
#   (diffvg.cpp:168-270 ignore shape_to_canvas).  Not compared.

def _linear(m):
    import torch
    return m.LinearGradient(begin=torch.tensor([8.0, 10.0]), end=torch.tensor([40.0, 36.0]),
                            offsets=torch.tensor([0.0, 0.45, 1.0]),
                            stop_colors=torch.tensor([[1.0, 0.0, 0.0, 1.0], [0.0, 1.0, 0.0, 0.8],
                                                      [0.0, 0.0, 1.0, 1.0]]))


def _radial(m):
    import torch
    return m.RadialGradient(center=torch.tensor([22.0, 26.0]), radius=torch.tensor([17.0, 12.0]),
                            offsets=torch.tensor([0.0, 0.6, 1.0]),
                            stop_colors=torch.tensor([[0.9, 0.8, 0.1, 1.0], [0.1, 0.3, 0.9, 0.7],
                                                      [0.6, 0.1, 0.2, 1.0]]))


def _paint(m, kind):
    import torch
    if kind == 'constant':
        return torch.tensor([0.2, 0.5, 0.9, 0.9])
    return _linear(m) if kind == 'linear' else _radial(m)


def loop_points(cx=24.0, cy=24.0, r=14.0):
    """A closed smooth loop of four cubic segments (a circle approximation)."""
    k = 0.5523 * r
    return [[cx + r, cy], [cx + r, cy + k], [cx + k, cy + r], [cx, cy + r], [cx - k, cy + r], [cx - r, cy + k],
            [cx - r, cy], [cx - r, cy - k], [cx - k, cy - r], [cx, cy - r], [cx + k, cy - r], [cx + r, cy - k]]


def paint_case(kind, stroke):
    """Builder of a 48x48, 2x2-spp scene: a rect filled with `kind` paint, or
    an open cubic path stroked with it (half width 3)."""
    def build(m):
        import torch
        if stroke:
            pts = torch.tensor([[6.0, 30.0], [14.0, 6.0], [30.0, 42.0], [42.0, 14.0]])
            shapes = [m.Path(num_control_points=torch.tensor([2], dtype=torch.int32), points=pts, is_closed=False,
                             stroke_width=torch.tensor(3.0))]
            groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_paint(m, kind))]
        else:
            shapes = [m.Rect(p_min=torch.tensor([4.0, 6.0]), p_max=torch.tensor([44.0, 42.0]))]
            groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_paint(m, kind))]
        return 48, 48, shapes, groups, False, 2
    build.__name__ = '%s_%s' % ('stroke' if stroke else 'fill', kind)
    return build


def transformed_gradient_stroke_case(m):
    """The closed loop stroked (half width 2.5) with a radial gradient, in a
    group with a rotated, scaled and translated shape_to_canvas; 4x4 spp."""
    import math
    import torch
    c, s = math.cos(0.3), math.sin(0.3)
    xf = torch.tensor([[1.1 * c, -0.9 * s, 2.0], [1.1 * s, 0.9 * c, -1.5], [0.0, 0.0, 1.0]])
    shapes = [m.Path(num_control_points=torch.full((4,), 2, dtype=torch.int32),
                     points=torch.tensor(loop_points()), is_closed=True, stroke_width=torch.tensor(2.5))]
    groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_radial(m),
                           shape_to_canvas=xf)]
    return 48, 48, shapes, groups, False, 4


def _paint_indices(packed, kind):
    """Arena offsets of the scene's one paint's parameters (for a radial
    gradient without its last stop's colour, see above)."""
    if kind == 'constant':
        co = slot_of(packed, 'color')
        return list(range(co, co + 4))
    gb = slot_of(packed, 'gradient_geometry')  # begin/end or center/radius
    so, sc = slot_of(packed, 'stop_offsets'), slot_of(packed, 'color')
    last = 8 if kind == 'radial' else 12
    return list(range(gb, gb + 4)) + list(range(so, so + 3)) + list(range(sc, sc + last))


def run_paint_checks(make_backend):
    """Paint parameters of constant / linear / radial paint on a fill and on a
    stroke (smooth at a fixed seed: one central difference, h = 1e-2), and a
    radial-gradient stroke in a transformed group: its paint parameters, and
    its stroke width through the boundary term (quarter-pixel steps averaged
    over 8 seeds).  Returns the relative errors by case name."""
    out = {}
    wts = weight_image(48, 48)
    for stroke in (False, True):
        for kind in ('constant', 'linear', 'radial'):
            builder = paint_case(kind, stroke)
            packed, P, fwd, bwd = make_backend(builder)
            idx = _paint_indices(packed, kind)
            g = analytic(bwd, P, wts, [3])
            fd = [central_fd(fwd, P, i, 1e-2, wts, [3]) for i in idx]
            out[builder.__name__] = rel_err(fd, g[idx])
    packed, P, fwd, bwd = make_backend(transformed_gradient_stroke_case)
    idx = _paint_indices(packed, 'radial')
    g = analytic(bwd, P, wts, [3])
    out['transformed_radial_stroke_paint'] = rel_err([central_fd(fwd, P, i, 1e-2, wts, [3]) for i in idx], g[idx])
    seeds = list(range(1, 9))
    sw = slot_of(packed, 'stroke_width')
    g = analytic(bwd, P, wts, seeds)
    out['transformed_radial_stroke_width'] = rel_err([central_fd(fwd, P, sw, 0.25, wts, seeds)], g[[sw]])
    return out


# ---------------------------------------------------------------------------
# Pixel filters.  The filter enters the gradients through gather_d_color
# (diffvg.cpp:777-815), for the interior and the boundary term alike, so the
# colour and geometry checks of run_checks are repeated under the tent, Hann
# and Gaussian filters (the Gaussian is not in the reference: these and the
# oracle parity test are its checks).  The filter radius's own gradient is
# not compared: the reference differentiates the normalised filter with
# (d.c ws - w d.c (ws - w)) / ws^2 (diffvg.cpp:1259-1262), which is not the
# derivative of sum(w c) / sum(w), and this project keeps that estimator.

def filter_case(ftype, radius):
    """Builder of the circle scene of circle_case rendered with pixel filter
    `ftype` of `radius` (attached as builder.filter), 48x48, 4x4 spp."""
    def build(m):
        return circle_case(m)
    build.filter = (ftype, radius)
    build.__name__ = 'filter_%s' % ftype
    return build


def run_filter_checks(make_backend):
    """Per filter (tent, Hann, Gaussian): the circle's colour gradient (one
    central difference, h = 1e-2) and its radius and centre through the
    boundary term (quarter-pixel steps averaged over 8 seeds)."""
    out = {}
    wts = weight_image(48, 48)
    seeds = list(range(1, 9))
    for ftype, radius in (('tent', 1.0), ('hann', 1.5), ('gaussian', 1.25)):
        packed, P, fwd, bwd = make_backend(filter_case(ftype, radius))
        co = slot_of(packed, 'color')
        g = analytic(bwd, P, wts, [1])
        out[ftype + '_color'] = rel_err([central_fd(fwd, P, co + k, 1e-2, wts, [1]) for k in range(4)], g[co:co + 4])
        ro, ce = slot_of(packed, 'radius'), slot_of(packed, 'center')
        idx = [ro, ce, ce + 1]
        g = analytic(bwd, P, wts, seeds)
        out[ftype + '_geometry'] = rel_err([central_fd(fwd, P, i, 0.25, wts, seeds) for i in idx], g[idx])
    return out
