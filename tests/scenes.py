"""Catalogue of small parity scenes: one per feature of the render path.

Every builder takes `mod`, a module with pydiffvg's scene classes (the
reference pydiffvg or diffvg_gb300), and returns a dict with the canvas,
shapes, groups and render settings.  The cases cover each shape kind, fill
and stroke, even-odd and non-zero rules, constant / linear / radial paints,
the four pixel filters, per-point thickness, group transforms, a background
image, prefiltering, distance-approximated quadratics, a render size that
differs from the canvas, and the signed-distance output.  Cases the
reference cannot run (gradient-coloured strokes crash it, ellipse strokes
and prefiltered circle strokes assert) are not in the catalogue.
"""
import math

import numpy as np
import torch


def _t(x):
    return torch.tensor(x, dtype=torch.float32)


def _case(w, h, shapes, groups, **kw):
    d = dict(canvas_width=w, canvas_height=h, shapes=shapes, groups=groups, width=w, height=h, spp=2, seed=7,
             filter=('box', 0.5), use_prefiltering=False, background=False, output='color', eval_positions=None)
    d.update(kw)
    return d


def star_points(cx, cy, r0, r1, n, phase=0.0):
    pts = []
    for k in range(2 * n):
        r = r0 if k % 2 == 0 else r1
        a = phase + math.pi * k / n
        pts.append([cx + r * math.cos(a), cy + r * math.sin(a)])
    return pts


def circle_fill(m):
    return _case(48, 48, [m.Circle(radius=_t(13.0), center=_t([22.0, 25.0]))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.3, 0.6, 0.3, 1.0]))])


def circle_stroke(m):
    return _case(48, 48, [m.Circle(radius=_t(14.0), center=_t([24.0, 23.0]), stroke_width=_t(2.5))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_t([0.9, 0.2, 0.1, 0.8]))])


def ellipse_fill(m):
    return _case(48, 48, [m.Ellipse(radius=_t([17.0, 9.0]), center=_t([24.0, 22.0]))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.2, 0.4, 0.9, 0.7]))])


def rect_fill_stroke(m):
    return _case(48, 48, [m.Rect(p_min=_t([8.5, 10.0]), p_max=_t([37.0, 33.5]), stroke_width=_t(1.5))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.8, 0.7, 0.1, 0.9]),
                               stroke_color=_t([0.1, 0.1, 0.6, 1.0]))])


def polygon_fill(m):
    pts = _t(star_points(24.0, 24.0, 19.0, 8.0, 5, 0.3))
    return _case(48, 48, [m.Polygon(points=pts, is_closed=True)],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.5, 0.1, 0.7, 1.0]),
                               use_even_odd_rule=False)])


def polygon_open_stroke(m):
    pts = _t([[5.0, 40.0], [15.0, 8.0], [27.0, 38.0], [42.0, 6.0]])
    return _case(48, 48, [m.Polygon(points=pts, is_closed=False, stroke_width=_t(2.0))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_t([0.0, 0.5, 0.5, 1.0]))])


def quadratic_fill_evenodd(m):
    # self-intersecting closed quadratic path: even-odd leaves a hole
    pts = _t([[6.0, 24.0], [24.0, -6.0], [42.0, 24.0], [24.0, 54.0], [10.0, 30.0], [24.0, 10.0],
              [38.0, 30.0], [24.0, 50.0]])
    ncp = torch.tensor([1, 1, 1, 1], dtype=torch.int32)
    return _case(48, 48, [m.Path(num_control_points=ncp, points=pts, is_closed=True)],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.9, 0.3, 0.2, 1.0]),
                               use_even_odd_rule=True)])


def quadratic_fill_nonzero(m):
    c = quadratic_fill_evenodd(m)
    c['groups'] = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.9, 0.3, 0.2, 1.0]),
                                use_even_odd_rule=False)]
    return c


def cubic_fill(m):
    pts = _t(star_points(24.0, 24.0, 18.0, 10.0, 6, 0.1))
    n = pts.shape[0] // 3
    pts = pts[:3 * n].contiguous()
    ncp = torch.full((n,), 2, dtype=torch.int32)
    return _case(48, 48, [m.Path(num_control_points=ncp, points=pts, is_closed=True)],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.2, 0.8, 0.4, 0.9]))])


def cubic_open_stroke(m):
    pts = _t([[4.0, 30.0], [12.0, 2.0], [22.0, 46.0], [30.0, 20.0], [36.0, 4.0], [44.0, 30.0], [40.0, 44.0]])
    ncp = torch.tensor([2, 2], dtype=torch.int32)
    return _case(48, 48, [m.Path(num_control_points=ncp, points=pts, is_closed=False, stroke_width=_t(2.2))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_t([0.7, 0.1, 0.9, 0.9]))])


def mixed_segments_fill_stroke(m):
    # line + quadratic + cubic in one closed path, filled and stroked
    pts = _t([[8.0, 8.0], [40.0, 8.0], [46.0, 24.0], [40.0, 40.0], [30.0, 48.0], [18.0, 30.0], [8.0, 40.0]])
    ncp = torch.tensor([0, 1, 2, 0], dtype=torch.int32)
    return _case(48, 48, [m.Path(num_control_points=ncp, points=pts, is_closed=True, stroke_width=_t(1.5))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.3, 0.3, 0.8, 0.6]),
                               stroke_color=_t([0.9, 0.9, 0.1, 1.0]), use_even_odd_rule=False)])


def thickness_stroke(m):
    pts = _t([[4.0, 24.0], [14.0, 4.0], [26.0, 44.0], [36.0, 24.0], [40.0, 10.0], [44.0, 30.0], [44.0, 44.0]])
    ncp = torch.tensor([2, 2], dtype=torch.int32)
    th = _t([1.0, 2.0, 3.0, 2.5, 1.5, 2.0, 1.0])
    return _case(48, 48, [m.Path(num_control_points=ncp, points=pts, is_closed=False, stroke_width=th)],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_t([0.1, 0.6, 0.2, 1.0]))])


def linear_gradient_fill(m):
    g = m.LinearGradient(begin=_t([8.0, 6.0]), end=_t([40.0, 42.0]), offsets=_t([0.0, 0.4, 1.0]),
                         stop_colors=_t([[1.0, 0.0, 0.0, 1.0], [0.0, 1.0, 0.0, 0.7], [0.0, 0.0, 1.0, 1.0]]))
    return _case(48, 48, [m.Circle(radius=_t(18.0), center=_t([24.0, 24.0]))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=g)])


def radial_gradient_fill(m):
    g = m.RadialGradient(center=_t([22.0, 26.0]), radius=_t([16.0, 12.0]), offsets=_t([0.1, 0.5, 0.9]),
                         stop_colors=_t([[1.0, 1.0, 0.0, 1.0], [0.0, 0.5, 1.0, 0.8], [0.5, 0.0, 0.5, 1.0]]))
    return _case(48, 48, [m.Rect(p_min=_t([4.0, 6.0]), p_max=_t([44.0, 42.0]))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=g)])


def transformed_group(m):
    a = 0.5
    xf = _t([[1.2 * math.cos(a), -0.8 * math.sin(a), 22.0], [1.2 * math.sin(a), 0.8 * math.cos(a), 20.0],
             [0.0, 0.0, 1.0]])
    pts = _t(star_points(0.0, 0.0, 14.0, 6.0, 4))
    return _case(48, 48, [m.Polygon(points=pts, is_closed=True, stroke_width=_t(1.2))],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.6, 0.2, 0.2, 1.0]),
                               stroke_color=_t([0.0, 0.0, 0.0, 1.0]), shape_to_canvas=xf)])


def multi_shape_group(m):
    shapes = [m.Circle(radius=_t(15.0), center=_t([20.0, 22.0])),
              m.Circle(radius=_t(10.0), center=_t([29.0, 26.0])),
              m.Rect(p_min=_t([6.0, 30.0]), p_max=_t([24.0, 44.0]))]
    return _case(48, 48, shapes,
                 [m.ShapeGroup(shape_ids=torch.tensor([0, 1, 2]), fill_color=_t([0.1, 0.5, 0.9, 1.0]),
                               use_even_odd_rule=True)])


def overlapping_groups(m):
    shapes = [m.Circle(radius=_t(14.0), center=_t([18.0, 20.0])),
              m.Rect(p_min=_t([16.0, 14.0]), p_max=_t([42.0, 40.0]), stroke_width=_t(2.0)),
              m.Polygon(points=_t([[4.0, 44.0], [24.0, 4.0], [44.0, 44.0]]), is_closed=True)]
    groups = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([1.0, 0.0, 0.0, 0.6])),
              m.ShapeGroup(shape_ids=torch.tensor([1]), fill_color=_t([0.0, 1.0, 0.0, 0.5]),
                           stroke_color=_t([0.0, 0.0, 0.0, 1.0])),
              m.ShapeGroup(shape_ids=torch.tensor([2]), fill_color=_t([0.0, 0.0, 1.0, 0.4]))]
    return _case(48, 48, shapes, groups)


def _with_filter(builder, ftype, radius):
    def f(m):
        c = builder(m)
        c['filter'] = (ftype, radius)
        return c
    f.__name__ = '%s_%s' % (builder.__name__, ftype)
    return f


def background_image(m):
    c = overlapping_groups(m)
    c['background'] = True
    return c


def render_size_differs(m):
    c = overlapping_groups(m)
    c['width'], c['height'] = 40, 56
    return c


def distance_approx_stroke(m):
    pts = _t([[4.0, 40.0], [20.0, 0.0], [30.0, 30.0], [40.0, 50.0], [44.0, 10.0]])
    ncp = torch.tensor([1, 1], dtype=torch.int32)
    return _case(48, 48, [m.Path(num_control_points=ncp, points=pts, is_closed=False, stroke_width=_t(2.0),
                                 use_distance_approx=True)],
                 [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=None, stroke_color=_t([0.4, 0.4, 0.0, 1.0]))])


def prefilter_fills(m):
    shapes, groups = [], []
    pts = _t(star_points(20.0, 22.0, 16.0, 9.0, 6, 0.2))
    n = pts.shape[0] // 3
    shapes.append(m.Path(num_control_points=torch.full((n,), 2, dtype=torch.int32), points=pts[:3 * n].contiguous(),
                         is_closed=True, stroke_width=_t(1.0)))
    groups.append(m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([0.9, 0.2, 0.2, 1.0]),
                               stroke_color=_t([0.1, 0.1, 0.1, 1.0])))
    shapes.append(m.Rect(p_min=_t([22.0, 18.0]), p_max=_t([44.0, 42.0])))
    groups.append(m.ShapeGroup(shape_ids=torch.tensor([1]),
                               fill_color=m.LinearGradient(begin=_t([22.0, 18.0]), end=_t([44.0, 42.0]),
                                                           offsets=_t([0.0, 1.0]),
                                                           stop_colors=_t([[0.0, 0.0, 1.0, 0.8],
                                                                           [0.0, 1.0, 1.0, 0.8]]))))
    shapes.append(m.Polygon(points=_t([[6.0, 44.0], [14.0, 28.0], [26.0, 46.0]]), is_closed=True))
    groups.append(m.ShapeGroup(shape_ids=torch.tensor([2]), fill_color=_t([0.2, 0.8, 0.2, 0.7])))
    return _case(48, 48, shapes, groups, use_prefiltering=True, spp=1)


def prefilter_strokes(m):
    c = cubic_open_stroke(m)
    c['use_prefiltering'] = True
    c['spp'] = 1
    return c


def prefilter_transformed_strokes(m):
    """Prefiltered strokes under rotated, anisotropically scaled group
    transforms; the second group strokes two shapes (a cubic and a rect)."""
    c = transformed_group(m)
    a = -0.3
    xf = _t([[0.9 * math.cos(a), -1.3 * math.sin(a), 26.0], [0.9 * math.sin(a), 1.3 * math.cos(a), 24.0],
             [0.0, 0.0, 1.0]])
    c['shapes'].append(m.Path(num_control_points=torch.tensor([2], dtype=torch.int32),
                              points=_t([[-14.0, 6.0], [-4.0, -16.0], [8.0, 14.0], [16.0, -6.0]]),
                              is_closed=False, stroke_width=_t(1.5)))
    c['shapes'].append(m.Rect(p_min=_t([-6.0, -5.0]), p_max=_t([7.0, 9.0]), stroke_width=_t(0.8)))
    c['groups'].append(m.ShapeGroup(shape_ids=torch.tensor([1, 2]), fill_color=None,
                                    stroke_color=_t([0.1, 0.3, 0.9, 0.9]), shape_to_canvas=xf))
    c['use_prefiltering'] = True
    c['spp'] = 1
    return c


def _long_fills(m):
    # closed star paths of 200-300 cubic segments (band lists), constant /
    # linear / radial fills, one in ten also stroked
    from diffvg_gb300 import workloads
    w, h, shapes, groups = workloads.fill_scene(m, seed=11, num_paths=8, canvas=96, seg_range=(200, 300),
                                                radius_range=(14.0, 44.0), stroke_fraction=0.25)
    return w, h, shapes, groups


def long_path_fills(m):
    w, h, shapes, groups = _long_fills(m)
    return _case(w, h, shapes, groups, spp=2, seed=5)


def long_path_fills_prefiltered(m):
    w, h, shapes, groups = _long_fills(m)
    return _case(w, h, shapes, groups, spp=1, seed=5, use_prefiltering=True)


def long_path_strokes(m):
    # open strokes of 120 cubic segments: more stroke records per group than
    # tile-mask bits
    from diffvg_gb300 import workloads
    w, h, shapes, groups = workloads.stroke_scene(m, seed=12, num_paths=6, canvas=96, step=4.0, num_segments=120,
                                                  width_range=(0.5, 2.0))
    return _case(w, h, shapes, groups, spp=2, seed=6)


def sdf_image(m):
    c = overlapping_groups(m)
    c['output'] = 'sdf'
    c['spp'] = 1
    # circles report "no closest point" in the reference; keep path and rect shapes only
    c['shapes'] = [m.Polygon(points=_t(star_points(20.0, 22.0, 14.0, 7.0, 5)), is_closed=True),
                   m.Rect(p_min=_t([16.0, 14.0]), p_max=_t([42.0, 40.0]))]
    c['groups'] = [m.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=_t([1.0, 0.0, 0.0, 1.0])),
                   m.ShapeGroup(shape_ids=torch.tensor([1]), fill_color=None, stroke_color=_t([0.0, 1.0, 0.0, 1.0]))]
    return c


def sdf_eval_positions(m):
    c = sdf_image(m)
    ev = (np.arange(200, dtype=np.float32).reshape(100, 2) * np.float32(0.23)) % np.float32(48.0)
    c['eval_positions'] = torch.from_numpy(ev.copy())
    return c


CASES = [circle_fill, circle_stroke, ellipse_fill, rect_fill_stroke, polygon_fill, polygon_open_stroke,
         quadratic_fill_evenodd, quadratic_fill_nonzero, cubic_fill, cubic_open_stroke, mixed_segments_fill_stroke,
         thickness_stroke, linear_gradient_fill, radial_gradient_fill, transformed_group, multi_shape_group,
         overlapping_groups, _with_filter(overlapping_groups, 'tent', 1.0),
         _with_filter(overlapping_groups, 'parabolic', 1.0), _with_filter(overlapping_groups, 'hann', 1.5),
         background_image, render_size_differs, distance_approx_stroke, prefilter_fills, prefilter_strokes,
         prefilter_transformed_strokes,
         sdf_image, sdf_eval_positions, long_path_fills, long_path_fills_prefiltered, long_path_strokes]

CASE_BY_NAME = {f.__name__: f for f in CASES}


def d_image_pattern(h, w, c, salt=0):
    """Deterministic adjoint image with values in {-1, -7/8, ..., 1}: integer
    arithmetic only, so it is bit-identical on every platform."""
    idx = np.arange(h * w * c, dtype=np.int64) + salt * 7919
    v = ((idx * 2654435761) % 17) - 8
    return (v.astype(np.float32) / np.float32(8.0)).reshape(h, w, c)


def background_pattern(h, w):
    y, x = np.meshgrid(np.arange(h, dtype=np.float32), np.arange(w, dtype=np.float32), indexing='ij')
    bg = np.stack([x / np.float32(w), y / np.float32(h), np.full_like(x, 0.5), np.full_like(x, 0.75)], axis=2)
    return bg.astype(np.float32)


def serialize(mod_render, m, case):
    """Flat argument list for `case` through `mod_render.RenderFunction`."""
    ftype, fr = case['filter']
    filt = m.PixelFilter(type=getattr(m_diffvg_enums(m).FilterType, ftype), radius=torch.tensor(fr))
    out_t = mod_render.OutputType.color if case['output'] == 'color' else mod_render.OutputType.sdf
    kw = dict(filter=filt, output_type=out_t, use_prefiltering=case['use_prefiltering'])
    if case['eval_positions'] is not None:
        kw['eval_positions'] = case['eval_positions']
    return mod_render.RenderFunction.serialize_scene(case['canvas_width'], case['canvas_height'], case['shapes'],
                                                     case['groups'], **kw)


def m_diffvg_enums(m):
    import sys
    if m.__name__ == 'pydiffvg':
        return sys.modules['diffvg']
    from diffvg_gb300 import diffvg
    return diffvg
