"""SVG file to scene: svg_to_scene(filename) -> (canvas_width, canvas_height,
shapes, shape_groups), with pydiffvg's semantics (pydiffvg/parse_svg.py).

Supported as there: <svg> width / height / viewBox; <g> with transform and
fill inheritance; <path>, <polygon>, <line>, <circle> and <rect>; <defs>,
<linearGradient> and <radialGradient> (with href inheritance, stops with
stop-color / stop-opacity, gradientTransform) and <style> class rules;
presentation attributes and the style attribute (fill, fill-opacity,
opacity, fill-rule, stroke, stroke-opacity, stroke-width, transform).
Stroke widths become half widths.  Colours: #rgb, #rrggbb, rgb(r, g, b),
url(#id), none and the CSS 2.1 colour keywords.

The reference's own behaviour is kept where it is observable from a scene:
<ellipse> is not read; a <rect> is placed at the origin with
p_max = (width, height) (parse_svg.py:488-500 never reads x / y);
a radial gradient's centre and radius stay at (0, 0) (parse_svg.py:201-263
passes its unset begin / end); fill opacity is written into the inherited
fill colour tensor, which the shapes that inherit it share.  The reference
depends on svgpathtools, cssutils and matplotlib for path data, style sheets
and colour names; path data is read by diffvg_gb300.svg_path, style sheets
by a small class-rule reader, colour names from a table.
"""
import re
import warnings
import xml.etree.ElementTree as etree

import numpy as np
import torch

from .shape import Circle, Path, Polygon, Rect, ShapeGroup, from_svg_path
from .color import LinearGradient, RadialGradient

__all__ = ['svg_to_scene', 'parse_scene', 'parse_color', 'parse_transform', 'parse_style', 'from_svg_path']

# CSS 2.1 colour keywords (sRGB, 0-255)
_NAMED = {
    'black': (0, 0, 0), 'silver': (192, 192, 192), 'gray': (128, 128, 128), 'grey': (128, 128, 128),
    'white': (255, 255, 255), 'maroon': (128, 0, 0), 'red': (255, 0, 0), 'purple': (128, 0, 128),
    'fuchsia': (255, 0, 255), 'magenta': (255, 0, 255), 'green': (0, 128, 0), 'lime': (0, 255, 0),
    'olive': (128, 128, 0), 'yellow': (255, 255, 0), 'navy': (0, 0, 128), 'blue': (0, 0, 255),
    'teal': (0, 128, 128), 'aqua': (0, 255, 255), 'cyan': (0, 255, 255), 'orange': (255, 165, 0),
}


def remove_namespaces(s):
    """'{namespace}tag' -> 'tag'."""
    return re.sub('{.*}', '', s)


def parse_style(s, defs):
    """'key: value; ...' -> dict; fill and stroke values become colours."""
    out = {}
    for item in s.split(';'):
        kv = item.split(':')
        if len(kv) == 2:
            key, value = kv[0].strip(), kv[1].strip()
            if key in ('fill', 'stroke'):
                value = parse_color(value, defs)
            out[key] = value
    return out


def parse_hex(s):
    s = s.lstrip('#')
    if len(s) == 3:
        s = ''.join(ch + ch for ch in s)
    return torch.tensor([int(s[k:k + 2], 16) / 255.0 for k in (0, 2, 4)])


def parse_int(s):
    """Integer part of a length, units dropped ('512px' -> 512)."""
    return int(float(''.join(ch for ch in s if not ch.isalpha())))


def parse_color(s, defs):
    """RGBA tensor, a gradient from defs, or None (parse_svg.py:54-80)."""
    if s is None:
        return None
    if isinstance(s, torch.Tensor):
        return s
    s = s.lstrip(' ')
    color = torch.tensor([0.0, 0.0, 0.0, 1.0])
    if s[0] == '#':
        color[:3] = parse_hex(s)
    elif s[:3] == 'url':
        color = defs[s[4:-1].lstrip('#')]
    elif s == 'none':
        color = None
    elif s[:4] == 'rgb(':
        rgb = s[4:-1].split(',')
        color = torch.tensor([int(rgb[0]) / 255.0, int(rgb[1]) / 255.0, int(rgb[2]) / 255.0, 1.0])
    elif s.strip().lower() in _NAMED:
        color = torch.tensor([c / 255.0 for c in _NAMED[s.strip().lower()]] + [1.0])
    else:
        warnings.warn('Unknown color command ' + s)
    return color


def _transform_item(item):
    kind, args = item.split('(')
    v = [float(x) for x in args.replace(',', ' ').split()]
    m = np.identity(3)
    if 'matrix' in kind:
        m[0, :] = [v[0], v[2], v[4]]
        m[1, :] = [v[1], v[3], v[5]]
    elif 'translate' in kind:
        m[0, 2] = v[0]
        if len(v) > 1:
            m[1, 2] = v[1]
    elif 'scale' in kind:
        m[0, 0] = v[0]
        m[1, 1] = v[1] if len(v) > 1 else v[0]
    elif 'rotate' in kind:
        a = np.radians(v[0])
        ox, oy = (v[1], v[2]) if len(v) == 3 else (0.0, 0.0)
        r = np.identity(3)
        r[:2, :2] = [[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]]
        to, back = np.identity(3), np.identity(3)
        to[:2, 2] = [ox, oy]
        back[:2, 2] = [-ox, -oy]
        m = to @ r @ back
    elif 'skewX' in kind:
        m[0, 1] = np.tan(np.radians(v[0]))
    elif 'skewY' in kind:
        m[1, 0] = np.tan(np.radians(v[0]))
    else:
        warnings.warn('Unknown SVG transform type: {0}'.format(kind))
    return m


def parse_transform(transform_str):
    """SVG transform list -> 3x3 float32 tensor (left to right products)."""
    if not transform_str:
        return np.identity(3)
    if not isinstance(transform_str, str):
        raise TypeError('Must provide a string to parse')
    m = np.identity(3)
    for item in transform_str.split(')')[:-1]:
        m = m @ _transform_item(item)
    return torch.from_numpy(m).type(torch.float32)


def _xform_point(m, p):
    q = m @ torch.cat((p, torch.ones([1])))
    return (q / q[2])[:2]


def _stops(node, defs, offsets, stop_colors):
    for child in node:
        if remove_namespaces(child.tag) != 'stop':
            continue
        color = [0.0, 0.0, 0.0, 1.0]
        if 'stop-color' in child.attrib:
            c = parse_color(child.attrib['stop-color'], defs)
            color[:3] = [c[0], c[1], c[2]]
        if 'stop-opacity' in child.attrib:
            color[3] = float(child.attrib['stop-opacity'])
        if 'style' in child.attrib:
            st = parse_style(child.attrib['style'], defs)
            if 'stop-color' in st:
                c = parse_color(st['stop-color'], defs)
                color[:3] = [c[0], c[1], c[2]]
            if 'stop-opacity' in st:
                color[3] = float(st['stop-opacity'])
        offsets.append(float(child.attrib['offset']))
        stop_colors.append(color)
    if isinstance(offsets, list):
        offsets = torch.tensor(offsets)
    if isinstance(stop_colors, list):
        stop_colors = torch.tensor(stop_colors)
    return offsets, stop_colors


def _inherited(node, defs):
    for key in node.attrib:
        if remove_namespaces(key) == 'href':
            return defs[node.attrib[key].lstrip('#')]
    return None


def parse_linear_gradient(node, transform, defs):
    begin, end = torch.tensor([0.0, 0.0]), torch.tensor([0.0, 0.0])
    offsets, stop_colors = [], []
    parent = _inherited(node, defs)
    if parent is not None:
        begin, end, offsets, stop_colors = parent.begin, parent.end, parent.offsets, parent.stop_colors
    for key in node.attrib:
        a = remove_namespaces(key)
        if a == 'x1':
            begin[0] = float(node.attrib['x1'])
        elif a == 'y1':
            begin[1] = float(node.attrib['y1'])
        elif a == 'x2':
            end[0] = float(node.attrib['x2'])
        elif a == 'y2':
            end[1] = float(node.attrib['y2'])
        elif a == 'gradientTransform':
            transform = transform @ parse_transform(node.attrib['gradientTransform'])
    begin, end = _xform_point(transform, begin), _xform_point(transform, end)
    offsets, stop_colors = _stops(node, defs, offsets, stop_colors)
    return LinearGradient(begin, end, offsets, stop_colors)


def parse_radial_gradient(node, transform, defs):
    # the reference reads cx / cy / fx / fy / fr but builds the gradient from
    # its unset begin / end (parse_svg.py:201-263): centre and radius (0, 0)
    begin, end = torch.tensor([0.0, 0.0]), torch.tensor([0.0, 0.0])
    offsets, stop_colors = [], []
    parent = _inherited(node, defs)
    if parent is not None:
        begin, end = getattr(parent, 'begin', begin), getattr(parent, 'end', end)
        offsets, stop_colors = parent.offsets, parent.stop_colors
    offsets, stop_colors = _stops(node, defs, offsets, stop_colors)
    return RadialGradient(begin, end, offsets, stop_colors)


def parse_stylesheet(node, transform, defs):
    """Class rules ('.name { key: value; ... }') of a <style> element."""
    text = node.text or ''
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    for sel, body in re.findall(r'([^{}]+)\{([^{}]*)\}', text):
        name = sel.strip()
        if len(name) >= 2 and name[0] == '.':
            defs[name[1:]] = parse_style(body, defs)
    return defs


def parse_defs(node, transform, defs):
    for child in node:
        tag = remove_namespaces(child.tag)
        if tag == 'linearGradient' and 'id' in child.attrib:
            defs[child.attrib['id']] = parse_linear_gradient(child, transform, defs)
        elif tag == 'radialGradient' and 'id' in child.attrib:
            defs[child.attrib['id']] = parse_radial_gradient(child, transform, defs)
        elif tag == 'style':
            defs = parse_stylesheet(child, transform, defs)
    return defs


def _half_width(v):
    if v[-2:] == 'px':
        v = v[:-2]
    return torch.tensor(float(v) / 2.0)


def _fill_rule(v, current):
    if v == 'evenodd':
        return True
    if v == 'nonzero':
        return False
    warnings.warn('Unknown fill-rule: {}'.format(v))
    return current


def parse_common_attrib(node, transform, fill_color, defs):
    """Transform, fill, stroke, half stroke width and fill rule of an element
    (parse_svg.py:288-387)."""
    attribs = {}
    if 'class' in node.attrib:
        attribs.update(defs[node.attrib['class']])
    attribs.update(node.attrib)
    stroke_color = None
    stroke_width = torch.tensor(0.5)
    even_odd = False
    new_transform = transform
    if 'transform' in attribs:
        new_transform = transform @ parse_transform(attribs['transform'])
    if 'fill' in attribs:
        fill_color = parse_color(attribs['fill'], defs)
    fill_opacity = 1.0
    if 'fill-opacity' in attribs:
        fill_opacity *= float(attribs['fill-opacity'])
    if 'opacity' in attribs:
        fill_opacity *= float(attribs['opacity'])
    if isinstance(fill_color, torch.Tensor):
        fill_color[3] = fill_opacity
    if 'fill-rule' in attribs:
        even_odd = _fill_rule(attribs['fill-rule'], even_odd)
    if 'stroke' in attribs:
        stroke_color = parse_color(attribs['stroke'], defs)
    if 'stroke-width' in attribs:
        stroke_width = _half_width(attribs['stroke-width'])
    if 'stroke-opacity' in attribs:
        stroke_color[3] = torch.tensor(float(attribs['stroke-opacity']))
    if 'style' in attribs:
        st = parse_style(attribs['style'], defs)
        if 'fill' in st:
            fill_color = parse_color(st['fill'], defs)
        fill_opacity = 1.0
        if 'fill-opacity' in st:
            fill_opacity *= float(st['fill-opacity'])
        if 'opacity' in st:
            fill_opacity *= float(st['opacity'])
        if 'fill-rule' in st:
            even_odd = _fill_rule(st['fill-rule'], even_odd)
        if isinstance(fill_color, torch.Tensor):
            fill_color[3] = fill_opacity
        if 'stroke' in st:
            # parse_style already turned 'none' into None, which replaces an
            # attribute's stroke here as in the reference
            stroke_color = parse_color(st['stroke'], defs)
            if isinstance(stroke_color, torch.Tensor):
                if 'stroke-opacity' in st:
                    stroke_color[3] = float(st['stroke-opacity'])
                if 'opacity' in st:
                    stroke_color[3] *= float(st['opacity'])
            if 'stroke-width' in st:
                stroke_width = _half_width(st['stroke-width'])
        for paint in (fill_color, stroke_color):
            if isinstance(paint, LinearGradient):
                paint.begin = _xform_point(new_transform, paint.begin)
                paint.end = _xform_point(new_transform, paint.end)
    return new_transform, fill_color, stroke_color, stroke_width, even_odd


def is_shape(tag):
    return tag in ('path', 'polygon', 'line', 'circle', 'rect')


def _group(shapes, shape_groups, new_shapes, fill, stroke, even_odd, xform, name, with_xform=True):
    first = len(shapes)
    shapes = shapes + new_shapes
    kw = dict(shape_ids=torch.tensor(list(range(first, len(shapes)))), fill_color=fill, stroke_color=stroke,
              use_even_odd_rule=even_odd, id=name)
    if with_xform:
        kw['shape_to_canvas'] = xform
    shape_groups.append(ShapeGroup(**kw))
    return shapes


def parse_shape(node, transform, fill_color, shapes, shape_groups, defs):
    """One shape element -> shapes and one group (parse_svg.py:392-516)."""
    tag = remove_namespaces(node.tag)
    xform, fill, stroke, width, even_odd = parse_common_attrib(node, transform, fill_color, defs)
    name = node.attrib.get('id', '')
    if tag == 'path':
        # the path's points are mapped to the canvas; its group keeps the identity
        paths = from_svg_path(node.attrib['d'], xform, fill is not None)
        for k, p in enumerate(paths):
            p.stroke_width = width
            p.source_id = name
            p.id = '{}-{}'.format(name, k) if len(paths) > 1 else name
        shapes = _group(shapes, shape_groups, paths, fill, stroke, even_odd, xform, name, with_xform=False)
    elif tag == 'polygon':
        # coordinates separated by spaces and / or commas, read in pairs (the
        # reference reads "x,y x,y ..." and "x y x y ..." the same way)
        nums = [float(v) for v in re.split(r'[\s,]+', node.attrib['points'].strip()) if v]
        poly = Polygon(torch.tensor(nums, dtype=torch.float32).view(-1, 2), fill is not None)
        poly.stroke_width = width
        shapes = _group(shapes, shape_groups, [poly], fill, stroke, even_odd, xform, name)
    elif tag == 'line':
        pts = torch.tensor([[float(node.attrib['x1']), float(node.attrib['y1'])],
                            [float(node.attrib['x2']), float(node.attrib['y2'])]])
        line = Polygon(pts, False)
        line.stroke_width = width
        shapes = _group(shapes, shape_groups, [line], fill, stroke, even_odd, xform, '')
    elif tag == 'circle':
        c = Circle(radius=torch.tensor(float(node.attrib['r'])),
                   center=torch.tensor([float(node.attrib['cx']), float(node.attrib['cy'])]))
        c.stroke_width = width
        shapes = _group(shapes, shape_groups, [c], fill, stroke, even_odd, xform, '')
    elif tag == 'rect':
        # parse_svg.py:488-500: x / y are never read and p_max = (x + w, x + h)
        x = y = 0.0
        w, h = float(node.attrib['width']), float(node.attrib['height'])
        r = Rect(p_min=torch.tensor([x, y]), p_max=torch.tensor([x + w, x + h]))
        r.stroke_width = width
        shapes = _group(shapes, shape_groups, [r], fill, stroke, even_odd, xform, '')
    return shapes, shape_groups


def parse_group(node, transform, fill_color, shapes, shape_groups, defs):
    if 'transform' in node.attrib:
        transform = transform @ parse_transform(node.attrib['transform'])
    if 'fill' in node.attrib:
        fill_color = parse_color(node.attrib['fill'], defs)
    for child in node:
        tag = remove_namespaces(child.tag)
        if is_shape(tag):
            shapes, shape_groups = parse_shape(child, transform, fill_color, shapes, shape_groups, defs)
        elif tag == 'g':
            shapes, shape_groups = parse_group(child, transform, fill_color, shapes, shape_groups, defs)
    return shapes, shape_groups


def parse_scene(node):
    """Root <svg> element -> (canvas_width, canvas_height, shapes, shape_groups)."""
    width = height = -1
    defs, shapes, shape_groups = {}, [], []
    fill_color = torch.tensor([0.0, 0.0, 0.0, 1.0])
    transform = torch.eye(3)
    if 'viewBox' in node.attrib:
        vb = node.attrib['viewBox'].split()
        width, height = parse_int(vb[2]), parse_int(vb[3])
    else:
        if 'width' in node.attrib:
            width = parse_int(node.attrib['width'])
        else:
            warnings.warn("Can't find canvas width.")
        if 'height' in node.attrib:
            height = parse_int(node.attrib['height'])
        else:
            warnings.warn("Can't find canvas height.")
    for child in node:
        tag = remove_namespaces(child.tag)
        if tag == 'defs':
            defs = parse_defs(child, transform, defs)
        elif tag == 'style':
            defs = parse_stylesheet(child, transform, defs)
        elif tag == 'linearGradient' and 'id' in child.attrib:
            defs[child.attrib['id']] = parse_linear_gradient(child, transform, defs)
        elif tag == 'radialGradient' and 'id' in child.attrib:
            defs[child.attrib['id']] = parse_radial_gradient(child, transform, defs)
        elif is_shape(tag):
            shapes, shape_groups = parse_shape(child, transform, fill_color, shapes, shape_groups, defs)
        elif tag == 'g':
            shapes, shape_groups = parse_group(child, transform, fill_color, shapes, shape_groups, defs)
    return width, height, shapes, shape_groups


def svg_to_scene(filename):
    """Load an SVG file as (canvas_width, canvas_height, shapes, shape_groups)."""
    return parse_scene(etree.parse(filename).getroot())
