"""Scene shape containers with pydiffvg's constructor signatures.

Reference: pydiffvg/shape.py:5-61.  These are plain records of tensors; the
renderer reads them through RenderFunction.serialize_scene.
``stroke_width`` is a half-width, as in the reference (within_distance.h:376).
For a Path, a stroke_width tensor with more than one element is a per-point
thickness (render_pytorch.py:67-72).
"""
import torch


class Circle:
    def __init__(self, radius, center, stroke_width=torch.tensor(1.0), id=''):
        self.radius = radius
        self.center = center
        self.stroke_width = stroke_width
        self.id = id


class Ellipse:
    def __init__(self, radius, center, stroke_width=torch.tensor(1.0), id=''):
        self.radius = radius
        self.center = center
        self.stroke_width = stroke_width
        self.id = id


class Path:
    def __init__(self, num_control_points, points, is_closed,
                 stroke_width=torch.tensor(1.0), id='', use_distance_approx=False):
        self.num_control_points = num_control_points
        self.points = points
        self.is_closed = is_closed
        self.stroke_width = stroke_width
        self.id = id
        self.use_distance_approx = use_distance_approx


class Polygon:
    def __init__(self, points, is_closed, stroke_width=torch.tensor(1.0), id=''):
        self.points = points
        self.is_closed = is_closed
        self.stroke_width = stroke_width
        self.id = id


class Rect:
    def __init__(self, p_min, p_max, stroke_width=torch.tensor(1.0), id=''):
        self.p_min = p_min
        self.p_max = p_max
        self.stroke_width = stroke_width
        self.id = id


class ShapeGroup:
    def __init__(self, shape_ids, fill_color, use_even_odd_rule=True,
                 stroke_color=None, shape_to_canvas=torch.eye(3), id=''):
        self.shape_ids = shape_ids
        self.fill_color = fill_color
        self.use_even_odd_rule = use_even_odd_rule
        self.stroke_color = stroke_color
        self.shape_to_canvas = shape_to_canvas
        self.id = id


def from_svg_path(path_str, shape_to_canvas=torch.eye(3), force_close=False):
    """Paths of an SVG path data string, one per continuous subpath
    (pydiffvg/shape.py:63-159).

    Lines, quadratic and cubic segments keep their points (0, 1 or 2 control
    points).  A subpath that ends where it starts is closed: when it was
    closed by a final line shorter than 1e-5 that line is dropped and the
    previous segment ends at the start; an open subpath whose ends are within
    1e-5 is closed the same way; otherwise force_close (set for filled shapes)
    adds a closing line.  Elliptical arcs become cubic segments of at most a
    quarter turn each (the control points of Cridge's "Bezier arcs"
    construction, as the reference uses; its intermediate end points are
    placed on the unrotated ellipse, as there).  Points are mapped through
    shape_to_canvas.
    """
    import math
    from . import svg_path as sp
    segs = sp.parse_path(path_str)
    if not segs:
        return []
    out = []
    for sub in sp.continuous_subpaths(segs):
        closed = sub[0].start == sub[-1].end
        if closed:
            if len(sub) > 1 and isinstance(sub[-1], sp.Line) and sub[-1].length() < 1e-5:
                sub = sub[:-1]
                sub[-1].end = sub[0].start
        else:
            beg, end = sub[0].start, sub[-1].end
            if abs(end - beg) < 1e-5:
                sub[-1].end = beg
                closed = True
            elif force_close:
                sub = sub + [sp.Line(end, beg)]
                closed = True
        ncp, pts = [], []
        for i, e in enumerate(sub):
            if i == 0:
                pts.append((e.start.real, e.start.imag))
            if isinstance(e, sp.Line):
                ncp.append(0)
            elif isinstance(e, sp.QuadraticBezier):
                ncp.append(1)
                pts.append((e.control.real, e.control.imag))
            elif isinstance(e, sp.CubicBezier):
                ncp.append(2)
                pts.append((e.control1.real, e.control1.imag))
                pts.append((e.control2.real, e.control2.imag))
            else:  # elliptical arc: cubic pieces of at most a quarter turn
                a0 = math.radians(e.theta)
                a1 = math.radians(e.theta + e.delta)
                sign = 1.0 if a1 >= a0 else -1.0
                rx, ry = e.radius.real, e.radius.imag
                cx, cy = e.center.real, e.center.imag
                rot = math.radians(e.phi)
                cr, sr = math.cos(rot), math.sin(rot)
                eps = 1e-5
                while sign * (a1 - a0) > eps:
                    step = a1 - a0
                    step = min(step, 0.5 * math.pi) if step > 0 else max(step, -0.5 * math.pi)
                    half = step / 2.0
                    ch, sh = math.cos(half), math.sin(half)
                    lam = (4.0 - ch) / 3.0
                    mu = sh + (ch - lam) / math.tan(half)
                    mid = a0 + half
                    cm, sm = math.cos(mid), math.sin(mid)
                    last = sign * (a1 - (a0 + step)) <= eps
                    ncp.append(2)
                    for (x, y) in ((lam * cm + mu * sm, lam * sm - mu * cm), (lam * cm - mu * sm, lam * sm + mu * cm)):
                        pts.append((cx + rx * (x * cr - y * sr), cy + ry * (x * sr + y * cr)))
                    if not last:
                        pts.append((cx + rx * math.cos(rot + a0 + step), cy + ry * math.sin(rot + a0 + step)))
                    a0 += step
            if i != len(sub) - 1 or not closed:
                pts.append((e.end.real, e.end.imag))
        p = torch.tensor(pts, dtype=torch.float32)
        p = torch.cat((p, torch.ones(p.shape[0], 1)), dim=1) @ torch.transpose(shape_to_canvas.to(torch.float32), 0, 1)
        p = (p / p[:, 2:3])[:, :2].contiguous()
        out.append(Path(torch.tensor(ncp, dtype=torch.int32), p, closed))
    return out
