"""Seeded synthetic scenes for the benchmark configurations.

The reference publishes no benchmark data; these generators produce scenes
with the sizes and value distributions of the five workload configurations
(plain small circle, stroke-heavy paths, fill-heavy prefiltered gradients,
batched mixed sizes, served requests).  Every generator takes `mod`, a module
with pydiffvg's scene classes (this package, or the reference pydiffvg), so
the same scene can be built for both implementations, and draws its random
numbers from a torch.Generator in the order documented in each function.
"""
import math

import torch


def _u(gen, *shape, lo=0.0, hi=1.0):
    return lo + (hi - lo) * torch.rand(*shape, generator=gen, dtype=torch.float32)


def circle_scene(mod, center=(128.0, 128.0), radius=40.0, color=(0.3, 0.6, 0.3, 1.0), canvas=256):
    """Config 1: one filled circle on a transparent canvas."""
    shapes = [mod.Circle(radius=torch.tensor(radius), center=torch.tensor(list(center)))]
    groups = [mod.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=torch.tensor(list(color)))]
    return canvas, canvas, shapes, groups


def stroke_scene(mod, seed=1, num_paths=2048, canvas=512, step=20.0, num_segments=4,
                 width_range=(1.0, 4.0)):
    """Config 2: open cubic paths, stroked, no fill.

    Draw order per path: first point U[0,canvas)^2, then 3*num_segments steps
    U[-step,step]^2 (cumulative), stroke half-width U[width_range], stroke
    RGBA U[0,1]^4."""
    gen = torch.Generator().manual_seed(seed)
    shapes, groups = [], []
    npts = 3 * num_segments + 1
    for i in range(num_paths):
        p0 = _u(gen, 2, hi=float(canvas))
        steps = _u(gen, npts - 1, 2, lo=-step, hi=step)
        pts = torch.cat([p0[None], p0[None] + torch.cumsum(steps, 0)], 0).contiguous()
        sw = _u(gen, 1, lo=width_range[0], hi=width_range[1])[0]
        col = _u(gen, 4)
        shapes.append(mod.Path(num_control_points=torch.full((num_segments,), 2, dtype=torch.int32),
                               points=pts, is_closed=False, stroke_width=sw))
        groups.append(mod.ShapeGroup(shape_ids=torch.tensor([i]), fill_color=None, stroke_color=col))
    return canvas, canvas, shapes, groups


def fill_scene(mod, seed=3, num_paths=512, canvas=1024, seg_range=(8, 32), radius_range=(10.0, 120.0),
               jitter=0.15, stroke_fraction=0.1, width_range=(0.5, 3.0)):
    """Config 3: closed star-shaped cubic paths with constant / linear / radial
    fills, a tenth also stroked (constant colour).

    Draw order per path: segment count U{seg_range}, centre U[0,canvas)^2,
    base radius U[radius_range], per-point jitter U[-jitter,jitter], then the
    fill paint (i%4 in {0,1}: RGBA U[0,1]^4; 2: linear c-R -> c+R with 3 stops
    of RGBA U[0,1]^4 at offsets 0, .5, 1; 3: radial at c, radius (R,R), same
    stops), then a stroke coin U[0,1) < stroke_fraction with half-width
    U[width_range] and RGBA U[0,1]^4."""
    gen = torch.Generator().manual_seed(seed)
    shapes, groups = [], []
    for i in range(num_paths):
        nseg = int(torch.randint(seg_range[0], seg_range[1] + 1, (1,), generator=gen)[0])
        c = _u(gen, 2, hi=float(canvas))
        R = float(_u(gen, 1, lo=radius_range[0], hi=radius_range[1])[0])
        n = 3 * nseg
        ang = torch.arange(n, dtype=torch.float32) * (2.0 * math.pi / n)
        rad = R * (1.0 + _u(gen, n, lo=-jitter, hi=jitter))
        pts = torch.stack([c[0] + rad * torch.cos(ang), c[1] + rad * torch.sin(ang)], 1).contiguous()
        shapes.append(mod.Path(num_control_points=torch.full((nseg,), 2, dtype=torch.int32),
                               points=pts, is_closed=True, stroke_width=torch.tensor(1.0)))
        kind = i % 4
        if kind in (0, 1):
            fill = _u(gen, 4)
        elif kind == 2:
            fill = mod.LinearGradient(begin=c - R, end=c + R, offsets=torch.tensor([0.0, 0.5, 1.0]),
                                      stop_colors=_u(gen, 3, 4))
        else:
            fill = mod.RadialGradient(center=c.clone(), radius=torch.tensor([R, R]),
                                      offsets=torch.tensor([0.0, 0.5, 1.0]), stop_colors=_u(gen, 3, 4))
        stroke = None
        if float(_u(gen, 1)[0]) < stroke_fraction:
            shapes[-1].stroke_width = _u(gen, 1, lo=width_range[0], hi=width_range[1])[0]
            stroke = _u(gen, 4)
        groups.append(mod.ShapeGroup(shape_ids=torch.tensor([i]), fill_color=fill, stroke_color=stroke))
    return canvas, canvas, shapes, groups


def blob_scene(mod, seed=5, num_paths=512, canvas=1024, seg_range=(8, 32), radius_range=(10.0, 120.0),
               lobes=(3, 7), amplitude=0.2, stroke_fraction=0.1, width_range=(0.5, 3.0)):
    """Closed smooth cubic paths of a chosen segment count: the same shape
    family whatever the count, for measuring how the cost per sample grows
    with the segments per path.

    Each path follows r(a) = R (1 + amplitude sin(k a + phase)) around its
    centre, cut into n cubic segments whose control points come from the
    curve's tangents (a C1 closed curve).  Draw order per path: n U{seg_range},
    centre U[0,canvas)^2, R U[radius_range], k U{lobes}, phase U[0, 2 pi),
    then the paints as in fill_scene (i%4 in {0,1}: RGBA U[0,1]^4; 2: linear,
    3: radial, 3 stops of RGBA U[0,1]^4 at offsets 0, .5, 1), then a stroke
    coin U[0,1) < stroke_fraction with half-width U[width_range] and RGBA
    U[0,1]^4."""
    gen = torch.Generator().manual_seed(seed)
    shapes, groups = [], []
    for i in range(num_paths):
        n = int(torch.randint(seg_range[0], seg_range[1] + 1, (1,), generator=gen)[0])
        c = _u(gen, 2, hi=float(canvas))
        R = float(_u(gen, 1, lo=radius_range[0], hi=radius_range[1])[0])
        k = int(torch.randint(lobes[0], lobes[1] + 1, (1,), generator=gen)[0])
        phase = float(_u(gen, 1, hi=2.0 * math.pi)[0])
        a = torch.arange(n, dtype=torch.float64) * (2.0 * math.pi / n)
        r = R * (1.0 + amplitude * torch.sin(k * a + phase))
        dr = R * amplitude * k * torch.cos(k * a + phase)
        p = torch.stack([c[0] + r * torch.cos(a), c[1] + r * torch.sin(a)], 1)
        # tangent per unit of a, scaled to one segment's span of a
        t = torch.stack([dr * torch.cos(a) - r * torch.sin(a), dr * torch.sin(a) + r * torch.cos(a)], 1)
        t = t * (2.0 * math.pi / n)
        nxt = torch.roll(torch.arange(n), -1)
        pts = torch.stack([p, p + t / 3.0, p[nxt] - t[nxt] / 3.0], 1).reshape(3 * n, 2).to(torch.float32)
        shapes.append(mod.Path(num_control_points=torch.full((n,), 2, dtype=torch.int32), points=pts.contiguous(),
                               is_closed=True, stroke_width=torch.tensor(1.0)))
        kind = i % 4
        cf = c.to(torch.float32)
        if kind in (0, 1):
            fill = _u(gen, 4)
        elif kind == 2:
            fill = mod.LinearGradient(begin=cf - R, end=cf + R, offsets=torch.tensor([0.0, 0.5, 1.0]),
                                      stop_colors=_u(gen, 3, 4))
        else:
            fill = mod.RadialGradient(center=cf.clone(), radius=torch.tensor([R, R]),
                                      offsets=torch.tensor([0.0, 0.5, 1.0]), stop_colors=_u(gen, 3, 4))
        stroke = None
        if float(_u(gen, 1)[0]) < stroke_fraction:
            shapes[-1].stroke_width = _u(gen, 1, lo=width_range[0], hi=width_range[1])[0]
            stroke = _u(gen, 4)
        groups.append(mod.ShapeGroup(shape_ids=torch.tensor([i]), fill_color=fill, stroke_color=stroke))
    return canvas, canvas, shapes, groups


def batched_scenes(mod, seeds=range(100, 164), canvases=(64, 128, 256, 512), path_range=(16, 1024)):
    """Config 4: independent stroke scenes of uneven size.

    Per scene (seed s): canvas U{canvases}, path count log-uniform in
    path_range, then stroke_scene(seed=s) with the step scaled by canvas/512."""
    out = []
    for s in seeds:
        gen = torch.Generator().manual_seed(int(s))
        canvas = canvases[int(torch.randint(0, len(canvases), (1,), generator=gen)[0])]
        lo, hi = math.log(path_range[0]), math.log(path_range[1])
        npaths = int(round(math.exp(lo + (hi - lo) * float(torch.rand(1, generator=gen)[0]))))
        out.append(stroke_scene(mod, seed=int(s) * 7919 + 1, num_paths=npaths, canvas=canvas,
                                step=20.0 * canvas / 512.0))
    return out


def perturbed_target_params(packed, params, seed, point_sigma=2.0, color_sigma=0.05):
    """Parameters of a batched-workload target: the scene's own parameters
    with points jittered by N(0, point_sigma^2) pixels and colours by
    N(0, color_sigma^2), colours clamped to [0, 1]."""
    gen = torch.Generator().manual_seed(int(seed) + 1000003)
    out = params.detach().cpu().clone()
    for sl in packed.slots:
        seg = out[sl.offset:sl.offset + sl.numel]
        if sl.kind == 'points':
            seg += point_sigma * torch.randn(sl.numel, generator=gen)
        elif sl.kind == 'color':
            seg.copy_((seg + color_sigma * torch.randn(sl.numel, generator=gen)).clamp_(0.0, 1.0))
    return out


def mixed_scene(mod, seed, canvas, num_paths):
    """Served-request scene: half open cubic strokes drawn like the
    stroke-heavy configuration (step scaled by canvas / 512), half closed
    star-shaped cubic fills with constant colours drawn like the fill-heavy
    configuration (radius range scaled by canvas / 1024)."""
    n_strokes = num_paths // 2
    w, h, s_shapes, s_groups = stroke_scene(mod, seed=seed, num_paths=n_strokes, canvas=canvas,
                                            step=20.0 * canvas / 512.0)
    _, _, f_shapes, f_groups = fill_scene(mod, seed=seed + 7, num_paths=num_paths - n_strokes, canvas=canvas,
                                          radius_range=(10.0 * canvas / 1024.0, 120.0 * canvas / 1024.0),
                                          stroke_fraction=0.0)
    shapes = s_shapes + f_shapes
    groups = list(s_groups)
    for k, g in enumerate(f_groups):
        fill = g.fill_color if isinstance(g.fill_color, torch.Tensor) else torch.rand(
            4, generator=torch.Generator().manual_seed(seed * 31 + k))
        groups.append(mod.ShapeGroup(shape_ids=torch.tensor([n_strokes + k]), fill_color=fill, stroke_color=None))
    return w, h, shapes, groups


def served_requests(mod, num_requests, seed0=500, canvases=(128, 256, 512), path_range=(64, 2048),
                    step_range=(100, 500)):
    """Request parameters of the served workload: per request (seed s)
    canvas U{canvases}, path count log-uniform in path_range, Adam step
    count U{step_range}; the target is a different seeded scene (seed
    s + 50000) of the same size."""
    out = []
    for r in range(num_requests):
        s = seed0 + r
        gen = torch.Generator().manual_seed(s)
        canvas = canvases[int(torch.randint(0, len(canvases), (1,), generator=gen)[0])]
        lo, hi = math.log(path_range[0]), math.log(path_range[1])
        npaths = int(round(math.exp(lo + (hi - lo) * float(torch.rand(1, generator=gen)[0]))))
        steps = int(torch.randint(step_range[0], step_range[1] + 1, (1,), generator=gen)[0])
        out.append(dict(seed=s, canvas=canvas, num_paths=npaths, steps=steps, target_seed=s + 50000))
    return out


def noisy_target(image, seed, sigma=0.02):
    """Target image: a render plus N(0, sigma^2) pixel noise."""
    gen = torch.Generator().manual_seed(int(seed))
    noise = sigma * torch.randn(tuple(image.shape), generator=gen)
    return image + noise.to(image.device)
