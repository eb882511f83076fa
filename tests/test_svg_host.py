"""SVG scene I/O (svg_to_scene, save_svg, from_svg_path and the path data
reader) on the CPU: the path data grammar, pydiffvg's subpath closing rules,
arcs as cubic pieces, the scene reader's attributes and the reference
behaviours it keeps, a save / load round trip, and a parsed scene rendered
by the oracle against the same scene built by hand."""

import numpy as np
import pytest
import torch

import diffvg_gb300 as dvg
from diffvg_gb300 import svg_path as sp


def _pts(path):
    return path.points.tolist()


def test_path_data_grammar():
    segs = sp.parse_path('M10-20L30.5.5e1l1e1,0')
    assert [type(s).__name__ for s in segs] == ['Line', 'Line']
    assert segs[0].start == complex(10, -20) and segs[0].end == complex(30.5, 5)
    assert segs[1].end == complex(40.5, 5)
    # a moveto's extra pairs are linetos; relative moveto at the start is absolute
    segs = sp.parse_path('m1 1 2 0 0 2z')
    assert [(s.start, s.end) for s in segs] == [(1 + 1j, 3 + 1j), (3 + 1j, 3 + 3j), (3 + 3j, 1 + 1j)]
    segs = sp.parse_path('M0 0 H5 v3 h-2 V0')
    assert [s.end for s in segs] == [5, 5 + 3j, 3 + 3j, 3]
    # S and T reflect the previous control point
    segs = sp.parse_path('M0 0 C1 2 3 2 4 0 S7 -2 8 0')
    assert segs[1].control1 == 5 - 2j
    segs = sp.parse_path('M0 0 Q1 2 2 0 T4 0')
    assert segs[1].control == 3 - 2j
    # arc flags without separators
    segs = sp.parse_path('M0 0a5 5 0 0010 0')
    assert isinstance(segs[0], sp.Arc) and segs[0].end == 10
    with pytest.raises(ValueError):
        sp.parse_path('L1 2')


def test_arc_centre_parameterisation():
    a = sp.parse_path('M0 0 A10 10 0 0 1 20 0')[0]
    assert a.center == pytest.approx(10 + 0j)
    assert a.theta == pytest.approx(180.0) and a.delta == pytest.approx(180.0)
    # radii too small for the chord are scaled up
    a = sp.parse_path('M0 0 A1 1 0 0 0 20 0')[0]
    assert a.radius.real == pytest.approx(10.0) and a.delta == pytest.approx(-180.0)


def test_subpath_closing_rules():
    # Z adds the closing line; the path is closed and keeps no duplicate point
    p, = dvg.from_svg_path('M10 20 L30 40 L50 20 Z')
    assert p.is_closed and p.num_control_points.tolist() == [0, 0, 0] and len(_pts(p)) == 3
    # a closing line shorter than 1e-5 is dropped
    p, = dvg.from_svg_path('M0 0 L10 0 L10 10 L0 0.000001 Z')
    assert p.is_closed and p.num_control_points.tolist() == [0, 0, 0]
    # an open path whose ends nearly meet is closed without a line
    p, = dvg.from_svg_path('M0 0 C5 0 10 5 10 10 C5 10 0 5 0.000001 0')
    assert p.is_closed and p.num_control_points.tolist() == [2, 2] and len(_pts(p)) == 6
    # force_close (filled shapes) adds a line; otherwise the path stays open
    p, = dvg.from_svg_path('M0 0 L10 0 L10 10', force_close=True)
    assert p.is_closed and p.num_control_points.tolist() == [0, 0, 0]
    p, = dvg.from_svg_path('M0 0 L10 0 L10 10')
    assert not p.is_closed and len(_pts(p)) == 3
    # two subpaths
    assert len(dvg.from_svg_path('M0 0 L1 0 M5 5 L6 5')) == 2
    # the shape-to-canvas transform maps the points
    xf = torch.tensor([[2.0, 0.0, 1.0], [0.0, 3.0, -1.0], [0.0, 0.0, 1.0]])
    p, = dvg.from_svg_path('M1 1 L2 2', xf)
    assert _pts(p) == [[3.0, 2.0], [5.0, 5.0]]


def test_arc_becomes_quarter_cubics_on_the_circle():
    p, = dvg.from_svg_path('M0 0 A10 10 0 1 1 0 20')   # a half turn on a circle of radius 10
    assert p.num_control_points.tolist() == [2, 2]
    pts = np.array(_pts(p), np.float64)
    c = np.array([0.0, 10.0])
    for k in range(2):
        b = pts[3 * k:3 * k + 4]
        for t in (0.25, 0.5, 0.75):
            q = ((1 - t) ** 3 * b[0] + 3 * (1 - t) ** 2 * t * b[1] + 3 * (1 - t) * t * t * b[2] + t ** 3 * b[3])
            assert abs(np.linalg.norm(q - c) - 10.0) < 3e-3       # cubic quarter arcs deviate < 3e-4 r


def _write(tmp_path, text):
    f = tmp_path / 'scene.svg'
    f.write_text(text)
    return str(f)


SAMPLE = '''<svg xmlns="http://www.w3.org/2000/svg" xmlns:xlink="http://www.w3.org/1999/xlink"
     width="64px" height="48">
  <defs>
    <linearGradient id="lg" x1="0" y1="0" x2="10" y2="0">
      <stop offset="0" stop-color="#ff0000"/>
      <stop offset="1" style="stop-color:blue;stop-opacity:0.5"/>
    </linearGradient>
    <linearGradient id="lg2" xlink:href="#lg" x2="20"/>
    <style>.thick { stroke: #00ff00; stroke-width: 4px }</style>
  </defs>
  <g transform="translate(5,6)" fill="#112233">
    <path d="M0 0 L10 0 L10 10 Z" opacity="0.5"/>
    <circle cx="20" cy="20" r="5" fill="url(#lg)" class="thick"/>
  </g>
  <polygon points="1,2 3,4 5,6" style="fill:none;stroke:red;stroke-width:2"/>
  <rect x="3" y="4" width="10" height="20" fill-rule="evenodd"/>
  <line x1="0" y1="0" x2="5" y2="5" stroke="black" transform="rotate(90)"/>
</svg>'''


def test_svg_to_scene_attributes(tmp_path):
    w, h, shapes, groups = dvg.svg_to_scene(_write(tmp_path, SAMPLE))
    assert (w, h) == (64, 48)
    assert [type(s).__name__ for s in shapes] == ['Path', 'Circle', 'Polygon', 'Rect', 'Polygon']
    # path points carry the group transform; its group keeps the identity
    assert _pts(shapes[0]) == [[5.0, 6.0], [15.0, 6.0], [15.0, 16.0]] and shapes[0].is_closed
    assert torch.equal(groups[0].shape_to_canvas, torch.eye(3))
    assert groups[0].fill_color.tolist() == pytest.approx([0x11 / 255, 0x22 / 255, 0x33 / 255, 0.5])
    # class style: stroke colour and half width; gradient fill; group transform on the group
    assert groups[1].stroke_color.tolist() == [0.0, 1.0, 0.0, 1.0]
    assert float(shapes[1].stroke_width) == 2.0
    lg = groups[1].fill_color
    assert isinstance(lg, dvg.LinearGradient)
    assert lg.offsets.tolist() == [0.0, 1.0]
    assert lg.stop_colors.tolist() == [[1.0, 0.0, 0.0, 1.0], [0.0, 0.0, 1.0, 0.5]]
    assert groups[1].shape_to_canvas[:2, 2].tolist() == [5.0, 6.0]
    # style: no fill, so the polygon stays open; named stroke colour
    assert groups[2].fill_color is None and not shapes[2].is_closed
    assert groups[2].stroke_color.tolist() == [1.0, 0.0, 0.0, 1.0] and float(shapes[2].stroke_width) == 1.0
    # the reference's rect: x / y unread, p_max = (x + w, x + h) with x = 0
    assert shapes[3].p_min.tolist() == [0.0, 0.0] and shapes[3].p_max.tolist() == [10.0, 20.0]
    assert groups[3].use_even_odd_rule
    # element transform on the line's group
    assert np.allclose(groups[4].shape_to_canvas[:2, :2].numpy(), [[0.0, -1.0], [1.0, 0.0]], atol=1e-6)


def test_gradient_href_inherits_stops(tmp_path):
    w, h, shapes, groups = dvg.svg_to_scene(_write(tmp_path, SAMPLE.replace('url(#lg)', 'url(#lg2)')))
    lg = groups[1].fill_color
    assert lg.end.tolist() == [20.0, 0.0]
    assert lg.stop_colors.tolist() == [[1.0, 0.0, 0.0, 1.0], [0.0, 0.0, 1.0, 0.5]]


def _scene():
    shapes = [dvg.Circle(radius=torch.tensor(10.0), center=torch.tensor([20.0, 22.0]), stroke_width=torch.tensor(1.5)),
              dvg.Path(num_control_points=torch.tensor([2, 2], dtype=torch.int32),
                       points=torch.tensor([[5.0, 5.0], [15.0, 0.0], [25.0, 10.0], [30.0, 20.0], [20.0, 30.0],
                                            [10.0, 25.0]]), is_closed=True, stroke_width=torch.tensor(0.5)),
              dvg.Polygon(points=torch.tensor([[1.0, 2.0], [30.0, 4.0], [5.0, 30.0]]), is_closed=True,
                          stroke_width=torch.tensor(1.0))]
    groups = [dvg.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=torch.tensor([0.2, 0.4, 0.6, 0.8]),
                             stroke_color=torch.tensor([1.0, 0.0, 0.0, 1.0])),
              dvg.ShapeGroup(shape_ids=torch.tensor([1]),
                             fill_color=dvg.LinearGradient(begin=torch.tensor([0.0, 0.0]), end=torch.tensor([10.0, 10.0]),
                                                           offsets=torch.tensor([0.0, 1.0]),
                                                           stop_colors=torch.tensor([[1.0, 0.0, 0.0, 1.0],
                                                                                     [0.0, 0.0, 1.0, 0.6]]))),
              dvg.ShapeGroup(shape_ids=torch.tensor([2]), fill_color=None, stroke_color=torch.tensor([0.0, 1.0, 0.0, 1.0]))]
    return shapes, groups


def test_save_load_round_trip(tmp_path):
    shapes, groups = _scene()
    f = str(tmp_path / 'out.svg')
    dvg.save_svg(f, 48, 40, shapes, groups)
    w, h, s2, g2 = dvg.svg_to_scene(f)
    assert (w, h) == (48, 40)
    assert [type(s).__name__ for s in s2] == ['Circle', 'Path', 'Polygon']
    assert float(s2[0].radius) == 10.0 and s2[0].center.tolist() == [20.0, 22.0]
    assert s2[1].num_control_points.tolist() == [2, 2] and s2[1].is_closed
    assert _pts(s2[1]) == _pts(shapes[1])
    assert _pts(s2[2]) == _pts(shapes[2])
    for a, b in zip(s2, shapes):
        assert float(a.stroke_width) == float(b.stroke_width)
    # colours go through rgb(0-255): within one step
    assert g2[0].fill_color.tolist() == pytest.approx(groups[0].fill_color.tolist(), abs=1 / 255)
    assert g2[0].stroke_color.tolist() == pytest.approx([1.0, 0.0, 0.0, 1.0])
    assert np.allclose(g2[1].fill_color.stop_colors.numpy(), groups[1].fill_color.stop_colors.numpy(), atol=1 / 255)
    assert g2[2].fill_color is None and g2[2].stroke_color.tolist() == [0.0, 1.0, 0.0, 1.0]


def test_parsed_scene_renders_like_the_hand_built_one(tmp_path):
    """A path and a polygon read from SVG feed the renderer the same
    parameters as the same scene built by hand (oracle, 32x32, 2x2 spp)."""
    import oracle
    from diffvg_gb300.packing import pack_scene
    svg = ('<svg xmlns="http://www.w3.org/2000/svg" width="32" height="32">'
           '<path d="M4 4 C12 0 28 8 26 16 Q20 30 6 24 Z" fill="#336699" stroke="#cc0000" stroke-width="2"/>'
           '<polygon points="2,30 16,18 30,30" fill="rgb(0,255,0)" opacity="0.5"/></svg>')
    w, h, shapes, groups = dvg.svg_to_scene(_write(tmp_path, svg))
    hand_shapes = [dvg.Path(num_control_points=torch.tensor([2, 1, 0], dtype=torch.int32),
                            points=torch.tensor([[4.0, 4.0], [12.0, 0.0], [28.0, 8.0], [26.0, 16.0], [20.0, 30.0],
                                                 [6.0, 24.0]]), is_closed=True, stroke_width=torch.tensor(1.0)),
                   dvg.Polygon(points=torch.tensor([[2.0, 30.0], [16.0, 18.0], [30.0, 30.0]]), is_closed=True,
                               stroke_width=torch.tensor(0.5))]
    hand_groups = [dvg.ShapeGroup(shape_ids=torch.tensor([0]),
                                  fill_color=torch.tensor([0x33 / 255, 0x66 / 255, 0x99 / 255, 1.0]),
                                  stroke_color=torch.tensor([0xcc / 255, 0.0, 0.0, 1.0])),
                   dvg.ShapeGroup(shape_ids=torch.tensor([1]), fill_color=torch.tensor([0.0, 1.0, 0.0, 0.5]))]
    imgs = []
    for sh, gr in ((shapes, groups), (hand_shapes, hand_groups)):
        packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, sh, gr))
        imgs.append(oracle.render(packed, oracle.params_of(packed), w, h, 2, 2, 5)['image'])
    assert np.array_equal(imgs[0], imgs[1])
    assert imgs[0][..., 3].max() > 0.9


def test_transforms_viewbox_and_inheritance(tmp_path):
    svg = ('<svg xmlns="http://www.w3.org/2000/svg" viewBox="0 0 40 30" width="400">'
           '<g fill="rgb(255,128,0)" transform="matrix(1 0 0 1 2 3)">'
           '<g transform="scale(2)"><path d="M0 0 L1 0 L1 1 Z M5 5 L6 5 L6 6 Z" stroke="#000" stroke-opacity="0.25"/></g>'
           '<polygon points="0 0,4 0 4,4" transform="skewX(45)"/></g>'
           '<circle cx="1" cy="2" r="3" fill="chartreuse"/></svg>')
    with pytest.warns(UserWarning):
        w, h, shapes, groups = dvg.svg_to_scene(_write(tmp_path, svg))
    assert (w, h) == (40, 30)                                   # the viewBox wins over width
    # one path element with two subpaths: two shapes in one group, points in canvas space
    assert groups[0].shape_ids.tolist() == [0, 1]
    assert _pts(shapes[0]) == [[2.0, 3.0], [4.0, 3.0], [4.0, 5.0]]
    assert _pts(shapes[1])[0] == [12.0, 13.0]
    assert groups[0].fill_color.tolist() == pytest.approx([1.0, 128 / 255, 0.0, 1.0])
    assert groups[0].stroke_color.tolist() == pytest.approx([0.0, 0.0, 0.0, 0.25])
    # the polygon's group carries matrix x skewX; its points stay local
    m = groups[1].shape_to_canvas.numpy()
    assert np.allclose(m, [[1.0, 1.0, 2.0], [0.0, 1.0, 3.0], [0.0, 0.0, 1.0]], atol=1e-6)
    assert _pts(shapes[2]) == [[0.0, 0.0], [4.0, 0.0], [4.0, 4.0]] and shapes[2].is_closed
    # an unknown colour name warns and stays black
    assert groups[2].fill_color.tolist() == [0.0, 0.0, 0.0, 1.0]


def test_save_svg_gamma_and_path_commands(tmp_path):
    shapes = [dvg.Path(num_control_points=torch.tensor([0, 1, 2], dtype=torch.int32),
                       points=torch.tensor([[0.0, 0.0], [4.0, 0.0], [6.0, 2.0], [4.0, 4.0], [2.0, 6.0], [0.0, 5.0]]),
                       is_closed=True)]
    groups = [dvg.ShapeGroup(shape_ids=torch.tensor([0]), fill_color=torch.tensor([0.0, 0.0, 1.0, 1.0]))]
    f = str(tmp_path / 'g.svg')
    dvg.save_svg(f, 8, 8, shapes, groups, use_gamma=True)
    text = open(f).read()
    assert 'feComponentTransfer' in text and 'filter:url(#gamma)' in text
    assert 'M 0.0 0.0 L 4.0 0.0 Q 6.0 2.0 4.0 4.0 C 2.0 6.0 0.0 5.0 0.0 0.0' in text
    w, h, s2, g2 = dvg.svg_to_scene(f)
    assert s2[0].num_control_points.tolist() == [0, 1, 2] and s2[0].is_closed
    assert _pts(s2[0]) == _pts(shapes[0])
