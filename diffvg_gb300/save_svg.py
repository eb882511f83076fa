"""Scene to SVG file: save_svg(filename, width, height, shapes, shape_groups,
use_gamma=False), with pydiffvg's output (pydiffvg/save_svg.py).

One element per shape group, drawn from the group's first shape: <circle>,
<polygon>, <path> (M / L / Q / C commands; a closed path's last segment ends
on its first point, so the file needs no Z), <rect> or <ellipse>; linear
gradients go to <defs> as shape_<i>_fill / shape_<i>_stroke; constant colours
are written as rgb(...) with the alpha in opacity / stroke-opacity; the
stroke width is written as a full width (twice the half width), with round
caps and joins.  use_gamma adds the reference's 1/2.2 gamma filter.
"""
import xml.etree.ElementTree as etree
from xml.dom import minidom

from .shape import Circle, Ellipse, Path, Polygon, Rect
from .color import LinearGradient

__all__ = ['save_svg']


def _num(x):
    return str(float(x))


def _rgb(c):
    return 'rgb({}, {}, {})'.format(int(255 * c[0]), int(255 * c[1]), int(255 * c[2]))


def _gamma_filter(defs):
    f = etree.SubElement(defs, 'filter', {'id': 'gamma', 'x': '0', 'y': '0', 'width': '100%', 'height': '100%'})
    tr = etree.SubElement(f, 'feComponentTransfer', {'color-interpolation-filters': 'sRGB'})
    for ch in 'RGBA':
        etree.SubElement(tr, 'feFunc' + ch, {'type': 'gamma', 'amplitude': '1', 'exponent': str(1 / 2.2)})


def _gradient(defs, paint, name):
    if not isinstance(paint, LinearGradient):
        return
    node = etree.SubElement(defs, 'linearGradient', {'id': name})
    node.set('x1', _num(paint.begin[0]))
    node.set('y1', _num(paint.begin[1]))
    node.set('x2', _num(paint.end[0]))
    node.set('y2', _num(paint.end[1]))
    offsets = paint.offsets.detach().cpu().numpy()
    colors = paint.stop_colors.detach().cpu().numpy()
    for j in range(offsets.shape[0]):
        etree.SubElement(node, 'stop', {'offset': str(offsets[j]), 'stop-color': _rgb(colors[j]),
                                        'stop-opacity': str(colors[j][3])})


def _path_data(shape):
    ncp = shape.num_control_points.detach().cpu().numpy()
    pts = shape.points.detach().cpu().numpy()
    n = pts.shape[0]
    out = ['M {} {}'.format(pts[0, 0], pts[0, 1])]
    k = 1
    for c in ncp:
        if c == 0:
            p = k % n
            out.append('L {} {}'.format(pts[p, 0], pts[p, 1]))
            k += 1
        elif c == 1:
            p = (k + 1) % n
            out.append('Q {} {} {} {}'.format(pts[k, 0], pts[k, 1], pts[p, 0], pts[p, 1]))
            k += 2
        else:
            p = (k + 2) % n
            out.append('C {} {} {} {} {} {}'.format(pts[k, 0], pts[k, 1], pts[k + 1, 0], pts[k + 1, 1],
                                                   pts[p, 0], pts[p, 1]))
            k += 3
    return ' '.join(out)


def _shape_node(parent, shape):
    if isinstance(shape, Circle):
        return etree.SubElement(parent, 'circle', {'r': _num(shape.radius), 'cx': _num(shape.center[0]),
                                                   'cy': _num(shape.center[1])})
    if isinstance(shape, Polygon):
        pts = shape.points.detach().cpu().numpy()
        return etree.SubElement(parent, 'polygon',
                                {'points': ' '.join('{} {}'.format(p[0], p[1]) for p in pts)})
    if isinstance(shape, Path):
        return etree.SubElement(parent, 'path', {'d': _path_data(shape)})
    if isinstance(shape, Rect):
        return etree.SubElement(parent, 'rect', {
            'x': _num(shape.p_min[0]), 'y': _num(shape.p_min[1]),
            'width': str(float(shape.p_max[0]) - float(shape.p_min[0])),
            'height': str(float(shape.p_max[1]) - float(shape.p_min[1]))})
    if isinstance(shape, Ellipse):
        return etree.SubElement(parent, 'ellipse', {'cx': _num(shape.center[0]), 'cy': _num(shape.center[1]),
                                                    'rx': _num(shape.radius[0]), 'ry': _num(shape.radius[1])})
    raise TypeError('save_svg: unsupported shape {}'.format(type(shape).__name__))


def save_svg(filename, width, height, shapes, shape_groups, use_gamma=False):
    root = etree.Element('svg', {'version': '1.1', 'xmlns': 'http://www.w3.org/2000/svg',
                                 'width': str(width), 'height': str(height)})
    defs = etree.SubElement(root, 'defs')
    g = etree.SubElement(root, 'g')
    if use_gamma:
        _gamma_filter(defs)
        g.set('style', 'filter:url(#gamma)')
    for i, grp in enumerate(shape_groups):
        if grp.fill_color is not None:
            _gradient(defs, grp.fill_color, 'shape_{}_fill'.format(i))
        if grp.stroke_color is not None:
            _gradient(defs, grp.stroke_color, 'shape_{}_stroke'.format(i))
    for i, grp in enumerate(shape_groups):
        shape = shapes[int(grp.shape_ids[0])]
        node = _shape_node(g, shape)
        node.set('stroke-width', str(2 * float(shape.stroke_width.detach().cpu().reshape(-1)[0])))
        fill = grp.fill_color
        if fill is None:
            node.set('fill', 'none')
        elif isinstance(fill, LinearGradient):
            node.set('fill', 'url(#shape_{}_fill)'.format(i))
        else:
            c = fill.detach().cpu().numpy()
            node.set('fill', _rgb(c))
            node.set('opacity', str(c[3]))
        stroke = grp.stroke_color
        if stroke is not None:
            if isinstance(stroke, LinearGradient):
                node.set('stroke', 'url(#shape_{}_stroke)'.format(i))
            else:
                c = stroke.detach().cpu().numpy()
                node.set('stroke', _rgb(c))
                node.set('stroke-opacity', str(c[3]))
            node.set('stroke-linecap', 'round')
            node.set('stroke-linejoin', 'round')
    text = minidom.parseString(etree.tostring(root, 'utf-8')).toprettyxml(indent='  ')
    with open(filename, 'w') as f:
        f.write(text)
