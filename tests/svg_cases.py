"""SVG documents for the scene-reader parity fixtures (tests/golden/svg_scenes.json)
and the helper that turns a parsed scene into plain lists for comparison."""

CASES = {
    'groups_styles_gradients': '''<svg xmlns="http://www.w3.org/2000/svg" xmlns:xlink="http://www.w3.org/1999/xlink"
     width="64px" height="48">
  <defs>
    <linearGradient id="lg" x1="0" y1="0" x2="10" y2="0">
      <stop offset="0" stop-color="#ff0000"/>
      <stop offset="1" style="stop-color:#0000ff;stop-opacity:0.5"/>
    </linearGradient>
    <style>.thick { stroke: #00ff00; stroke-width: 4px }</style>
  </defs>
  <g transform="translate(5,6)" fill="#112233">
    <path d="M0 0 L10 0 L10 10 Z" opacity="0.5"/>
    <circle cx="20" cy="20" r="5" fill="url(#lg)" class="thick"/>
  </g>
  <polygon points="1,2 3,4 5,6" style="fill:none;stroke:#ff0000;stroke-width:2"/>
  <rect x="3" y="4" width="10" height="20" fill-rule="evenodd" fill="#00ff00"/>
  <line x1="0" y1="0" x2="5" y2="5" stroke="#000000" transform="rotate(90)" fill="#ffffff"/>
</svg>''',
    'path_commands': '''<svg xmlns="http://www.w3.org/2000/svg" width="100" height="80">
  <path d="M10 10 C20 0 30 0 40 10 S60 20 70 10 Q80 0 90 10 T90 30 L90 50 H60 V70 Z"
        fill="#336699" stroke="#cc0000" stroke-width="1.5" stroke-opacity="0.7"/>
  <path d="m5 60 l10 0 0 10 -10 0 z m20 0 h10 v10 h-10 z" fill="#808080" fill-opacity="0.4"/>
  <path d="M40 40 C45 35 50 35 55 40" fill="none" stroke="#ff00ff" style="stroke-width:3px;opacity:0.5"/>
</svg>''',
    'arcs': '''<svg xmlns="http://www.w3.org/2000/svg" width="64" height="64">
  <path d="M10 32 A22 22 0 0 1 54 32 A22 22 0 0 1 10 32 Z" fill="#ff8000"/>
  <path d="M5 5 a10 5 30 1 0 20 10" fill="none" stroke="#000080"/>
</svg>''',
    'transforms_viewbox': '''<svg xmlns="http://www.w3.org/2000/svg" viewBox="0 0 40 30" width="400">
  <g fill="rgb(255,128,0)" transform="matrix(1 0 0 1 2 3)">
    <g transform="scale(2)"><path d="M0 0 L1 0 L1 1 Z M5 5 L6 5 L6 6 Z" stroke="#000" stroke-opacity="0.25"/></g>
    <polygon points="0,0 4,0 4,4" transform="skewX(30) translate(1 2)"/>
  </g>
  <g transform="rotate(30 10 10)" fill="#00ffff">
    <circle cx="10" cy="10" r="4" style="fill:#ff00ff;fill-opacity:0.5;stroke:#000000;stroke-width:1"/>
  </g>
</svg>''',
    'inheritance_and_opacity': '''<svg xmlns="http://www.w3.org/2000/svg" xmlns:xlink="http://www.w3.org/1999/xlink"
     width="50" height="40">
  <radialGradient id="rg" cx="5" cy="5" r="3">
    <stop offset="0" stop-color="red"/>
    <stop offset="0.5" stop-color="navy" stop-opacity="0.3"/>
    <stop offset="1" style="stop-color:#0f0"/>
  </radialGradient>
  <linearGradient id="base" x1="1" y1="2" x2="3" y2="4">
    <stop offset="0" stop-color="#fff"/><stop offset="1" stop-color="#000"/>
  </linearGradient>
  <linearGradient id="derived" xlink:href="#base" x2="9" gradientTransform="translate(1,1)"/>
  <style>.c1 { fill: #204060; fill-opacity: 0.5 } .c2 { stroke: #abcdef; stroke-width: 3 }</style>
  <g fill="#808000" transform="translate(2,3)">
    <path d="M1 1 L9 1 L9 9 Z" fill-opacity="0.25"/>
    <path d="M11 1 L19 1 L19 9 Z"/>
    <circle cx="30" cy="10" r="4" class="c1"/>
    <circle cx="40" cy="10" r="4" class="c2" fill="url(#derived)" style="stroke:#123456;stroke-width:2"/>
    <circle cx="45" cy="30" r="3" fill="url(#rg)" stroke="navy"/>
  </g>
  <rect width="5" height="6" style="fill:teal;opacity:0.5;stroke:black;stroke-opacity:0.4"
        transform="translate(10 20)"/>
  <path d="M20 20 L30 20 L30 30 Z" fill="url(#derived)" style="stroke:#ff0000"/>
</svg>''',
}


def _t(x):
    return [float(v) for v in x.detach().reshape(-1).tolist()]


def _paint(p):
    if p is None:
        return None
    name = type(p).__name__
    if name == 'LinearGradient':
        return {'kind': 'linear', 'begin': _t(p.begin), 'end': _t(p.end), 'offsets': _t(p.offsets),
                'stop_colors': _t(p.stop_colors)}
    if name == 'RadialGradient':
        return {'kind': 'radial', 'center': _t(p.center), 'radius': _t(p.radius), 'offsets': _t(p.offsets),
                'stop_colors': _t(p.stop_colors)}
    return {'kind': 'constant', 'rgba': _t(p)}


def describe(width, height, shapes, groups):
    """Plain lists of a parsed scene (shape parameters, group paints and transforms)."""
    out = {'width': width, 'height': height, 'shapes': [], 'groups': []}
    for s in shapes:
        name = type(s).__name__
        d = {'type': name, 'stroke_width': _t(s.stroke_width)}
        if name in ('Path',):
            d.update(num_control_points=[int(v) for v in s.num_control_points.tolist()], points=_t(s.points),
                     is_closed=bool(s.is_closed))
        elif name == 'Polygon':
            d.update(points=_t(s.points), is_closed=bool(s.is_closed))
        elif name == 'Circle':
            d.update(radius=_t(s.radius), center=_t(s.center))
        elif name == 'Rect':
            d.update(p_min=_t(s.p_min), p_max=_t(s.p_max))
        out['shapes'].append(d)
    for g in groups:
        out['groups'].append({'shape_ids': [int(v) for v in g.shape_ids.tolist()], 'fill': _paint(g.fill_color),
                              'stroke': _paint(g.stroke_color), 'even_odd': bool(g.use_even_odd_rule),
                              'shape_to_canvas': _t(g.shape_to_canvas)})
    return out


def save_scenes(m):
    """Scenes for the writer's parity fixtures, built with module m's classes:
    name -> (width, height, shapes, shape_groups, use_gamma)."""
    import torch
    t = torch.tensor
    shapes = [m.Circle(radius=t(10.0), center=t([20.0, 22.0]), stroke_width=t(1.5)),
              m.Path(num_control_points=t([0, 1, 2], dtype=torch.int32),
                     points=t([[0.0, 0.0], [4.0, 0.0], [6.0, 2.0], [4.0, 4.0], [2.0, 6.0], [0.0, 5.0]]),
                     is_closed=True, stroke_width=t(0.5)),
              m.Polygon(points=t([[1.0, 2.0], [30.0, 4.0], [5.0, 30.0]]), is_closed=True, stroke_width=t(1.0)),
              m.Rect(p_min=t([3.0, 4.0]), p_max=t([13.0, 24.0]), stroke_width=t(2.0)),
              m.Ellipse(radius=t([6.0, 3.0]), center=t([30.0, 10.0]))]
    groups = [m.ShapeGroup(shape_ids=t([0]), fill_color=t([0.2, 0.4, 0.6, 0.8]), stroke_color=t([1.0, 0.0, 0.0, 1.0])),
              m.ShapeGroup(shape_ids=t([1]),
                           fill_color=m.LinearGradient(begin=t([0.0, 0.0]), end=t([10.0, 10.0]), offsets=t([0.0, 1.0]),
                                                       stop_colors=t([[1.0, 0.0, 0.0, 1.0], [0.0, 0.0, 1.0, 0.5]]))),
              m.ShapeGroup(shape_ids=t([2]), fill_color=None, stroke_color=t([0.0, 1.0, 0.0, 1.0])),
              m.ShapeGroup(shape_ids=t([3]), fill_color=t([0.5, 0.5, 0.5, 1.0])),
              m.ShapeGroup(shape_ids=t([4]), fill_color=t([0.1, 0.9, 0.3, 0.6]))]
    return {'plain': (48, 40, shapes, groups, False), 'gamma': (48, 40, shapes[:2], groups[:2], True)}
