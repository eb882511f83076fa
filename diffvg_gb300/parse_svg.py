"""SVG file to scene: svg_to_scene(filename) -> (canvas_width, canvas_height,
shapes, shape_groups), with the semantics of pydiffvg's reader
(pydiffvg/parse_svg.py).

The reader works in two steps per element.  A style resolution step folds
the element's presentation (its class rule, then its own attributes) and its
inline style attribute into one resolved record: transform, fill paint,
stroke paint, half stroke width, fill rule.  An emission step turns the
element and that record into shapes and one shape group.  Paint servers
(<linearGradient>, <radialGradient>) and class rules (<style>) live in one
registry filled in document order.

Read as in pydiffvg: <svg> width / height / viewBox; <g> transform and fill
(the only attributes a group passes down); <path>, <polygon>, <line>,
<circle>, <rect>; gradients and style sheets at the top level or in <defs>;
presentation attributes and the style attribute (fill, fill-opacity,
opacity, fill-rule, stroke, stroke-opacity, stroke-width, transform).
Stroke widths become half widths.  Colours: #rgb, #rrggbb, rgb(r, g, b),
url(#id), none and the CSS 2.1 colour keywords.

pydiffvg's observable behaviour is kept, including where it departs from
SVG: <ellipse> is not read; a <rect> sits at the origin with p_max =
(width, height) (its x / y are ignored, parse_svg.py:488-500); a radial
gradient's centre and radius stay (0, 0) unless inherited
(parse_svg.py:201-263); opacities are written into the paint tensor that an
element inherits, which every element sharing it sees; the inline style's
opacities replace the attributes' ones; an inline style moves every linear
gradient the element uses by the element's transform, in place on the
shared gradient.  pydiffvg reads path data, style sheets and colour names
through svgpathtools, cssutils and matplotlib; here path data is read by
diffvg_gb300.svg_path, style sheets by a class-rule reader and colour names
from a table.
"""
from dataclasses import dataclass
import math
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

_SHAPE_TAGS = frozenset(('path', 'polygon', 'line', 'circle', 'rect'))


def _tag(element):
    """Element name without its namespace."""
    return element.tag.rpartition('}')[2]


def _attr(element, local_name):
    """Value of an attribute by local name (any namespace), or None."""
    for key, value in element.attrib.items():
        if key.rpartition('}')[2] == local_name:
            return value
    return None


# --------------------------------------------------------------------------
# values

def _declarations(text):
    """'name: value; ...' -> {name: value} (entries without exactly one ':'
    are dropped)."""
    out = {}
    for entry in text.split(';'):
        parts = entry.split(':')
        if len(parts) == 2:
            out[parts[0].strip()] = parts[1].strip()
    return out


def parse_style(s, defs):
    """A style declaration list as a dict; fill and stroke values are read as
    paints through `defs` (parse_svg.py:24-35)."""
    out = _declarations(s)
    for name in ('fill', 'stroke'):
        if name in out:
            out[name] = parse_color(out[name], defs)
    return out


def _rgb_hex(digits):
    if len(digits) == 3:
        digits = ''.join(2 * d for d in digits)
    return [int(digits[k:k + 2], 16) / 255.0 for k in range(0, 6, 2)]


def parse_color(s, defs):
    """A paint value: an RGBA tensor, a gradient registered in `defs`, or None
    for 'none' (parse_svg.py:54-80).  An unknown value warns and gives opaque
    black; a value that is already a tensor is returned as it is."""
    if s is None or isinstance(s, torch.Tensor):
        return s
    text = s.lstrip(' ')
    if text.startswith('url'):
        return defs[text[4:-1].lstrip('#')]
    if text == 'none':
        return None
    rgba = [0.0, 0.0, 0.0, 1.0]
    if text.startswith('#'):
        rgba[:3] = _rgb_hex(text[1:])
    elif text.startswith('rgb('):
        rgba[:3] = [int(v) / 255.0 for v in text[4:-1].split(',')[:3]]
    elif text.strip().lower() in _NAMED:
        rgba[:3] = [v / 255.0 for v in _NAMED[text.strip().lower()]]
    else:
        warnings.warn('Unknown color command ' + s)
    return torch.tensor(rgba)


def _length(s):
    """Integer part of a length with its unit letters dropped ('64px' -> 64)."""
    return int(float(''.join(ch for ch in s if not ch.isalpha())))


def _half_width(s):
    """Half of a stroke-width value (pydiffvg stores half widths)."""
    return torch.tensor(float(s[:-2] if s.endswith('px') else s) / 2.0)


def _even_odd(value, current):
    rules = {'evenodd': True, 'nonzero': False}
    if value not in rules:
        warnings.warn('Unknown fill-rule: {}'.format(value))
        return current
    return rules[value]


# --------------------------------------------------------------------------
# transforms

def _affine(a, b, c, d, e, f):
    return np.array([[a, c, e], [b, d, f], [0.0, 0.0, 1.0]])


def _rotation(deg, cx=0.0, cy=0.0):
    t = math.radians(deg)
    co, si = math.cos(t), math.sin(t)
    # about (cx, cy): translate(cx, cy) rotate(deg) translate(-cx, -cy)
    return _affine(1, 0, 0, 1, cx, cy) @ _affine(co, si, -si, co, 0, 0) @ _affine(1, 0, 0, 1, -cx, -cy)


_TRANSFORMS = {
    'matrix': lambda v: _affine(*v[:6]),
    'translate': lambda v: _affine(1, 0, 0, 1, v[0], v[1] if len(v) > 1 else 0.0),
    'scale': lambda v: _affine(v[0], 0, 0, v[1] if len(v) > 1 else v[0], 0, 0),
    'rotate': lambda v: _rotation(v[0], *(v[1:3] if len(v) == 3 else ())),
    'skewX': lambda v: _affine(1, 0, math.tan(math.radians(v[0])), 1, 0, 0),
    'skewY': lambda v: _affine(1, math.tan(math.radians(v[0])), 0, 1, 0, 0),
}


def parse_transform(transform_str):
    """An SVG transform list as a 3x3 float32 tensor, the product of its
    items from left to right (parse_svg.py:82-135).  An empty string gives
    the identity (as a float64 array, as pydiffvg returns it)."""
    if not transform_str:
        return np.identity(3)
    if not isinstance(transform_str, str):
        raise TypeError('Must provide a string to parse')
    m = np.identity(3)
    for item in transform_str.split(')')[:-1]:
        name, _, args = item.partition('(')
        values = [float(x) for x in args.replace(',', ' ').split()]
        kind = next((k for k in _TRANSFORMS if k in name), None)
        if kind is None:
            warnings.warn('Unknown SVG transform type: {0}'.format(name))
            continue
        m = m @ _TRANSFORMS[kind](values)
    return torch.from_numpy(m).type(torch.float32)


def _apply(m, p):
    """A 2-D point through a 3x3 (projective) transform."""
    q = m @ torch.cat((p, torch.ones([1])))
    return (q / q[2])[:2]


# --------------------------------------------------------------------------
# paint servers and class rules

def _stops(element, defs, inherited):
    """Offsets and colours of the <stop> children.  A gradient with an href
    keeps its parent's stop tensors; pydiffvg cannot add stops of its own to
    those (it appends to the tensors), and neither can this reader."""
    own = [s for s in element if _tag(s) == 'stop']
    if inherited is not None:
        if own:
            raise ValueError('a gradient with an href cannot add <stop> elements to its parent\'s stops')
        return inherited
    offsets, colors = [], []
    for stop in own:
        rgba = [0.0, 0.0, 0.0, 1.0]
        decl = {'stop-color': stop.attrib.get('stop-color'), 'stop-opacity': stop.attrib.get('stop-opacity')}
        if 'style' in stop.attrib:
            style = parse_style(stop.attrib['style'], defs)
            decl.update({k: style[k] for k in ('stop-color', 'stop-opacity') if k in style})
        if decl['stop-color'] is not None:
            c = parse_color(decl['stop-color'], defs)
            rgba[:3] = [c[0], c[1], c[2]]
        if decl['stop-opacity'] is not None:
            rgba[3] = float(decl['stop-opacity'])
        offsets.append(float(stop.attrib['offset']))
        colors.append(rgba)
    return torch.tensor(offsets), torch.tensor(colors)


def _linear_gradient(element, defs):
    """parse_svg.py:137-199: x1 / y1 / x2 / y2 written into the (possibly
    inherited) end-point tensors, then gradientTransform applied."""
    parent = defs[_attr(element, 'href').lstrip('#')] if _attr(element, 'href') is not None else None
    begin = parent.begin if parent is not None else torch.tensor([0.0, 0.0])
    end = parent.end if parent is not None else torch.tensor([0.0, 0.0])
    for name, (vec, k) in (('x1', (begin, 0)), ('y1', (begin, 1)), ('x2', (end, 0)), ('y2', (end, 1))):
        value = _attr(element, name)
        if value is not None:
            vec[k] = float(value)
    m = torch.eye(3)
    if _attr(element, 'gradientTransform') is not None:
        m = m @ parse_transform(_attr(element, 'gradientTransform'))
    offsets, colors = _stops(element, defs, (parent.offsets, parent.stop_colors) if parent is not None else None)
    return LinearGradient(_apply(m, begin), _apply(m, end), offsets, colors)


def _radial_gradient(element, defs):
    """parse_svg.py:201-263 reads cx / cy / r but builds the gradient from its
    unset begin / end: centre and radius are (0, 0), or the end points of an
    inherited linear gradient."""
    parent = defs[_attr(element, 'href').lstrip('#')] if _attr(element, 'href') is not None else None
    center = getattr(parent, 'begin', torch.tensor([0.0, 0.0]))
    radius = getattr(parent, 'end', torch.tensor([0.0, 0.0]))
    offsets, colors = _stops(element, defs, (parent.offsets, parent.stop_colors) if parent is not None else None)
    return RadialGradient(center, radius, offsets, colors)


def _class_rules(element, defs):
    """Class rules ('.name { declarations }') of a <style> element."""
    text = re.sub(r'/\*.*?\*/', '', element.text or '', flags=re.S)
    for selector, body in re.findall(r'([^{}]+)\{([^{}]*)\}', text):
        selector = selector.strip()
        if len(selector) > 1 and selector.startswith('.'):
            defs[selector[1:]] = parse_style(body, defs)


def _register(element, defs):
    """Adds a definition element (gradient with an id, or style sheet) to
    `defs`; returns whether the element was one."""
    tag = _tag(element)
    if tag == 'style':
        _class_rules(element, defs)
    elif tag in ('linearGradient', 'radialGradient'):
        if 'id' in element.attrib:
            build = _linear_gradient if tag == 'linearGradient' else _radial_gradient
            defs[element.attrib['id']] = build(element, defs)
    else:
        return False
    return True


# --------------------------------------------------------------------------
# style resolution

@dataclass
class _Resolved:
    transform: object
    fill: object
    stroke: object = None
    half_width: object = None
    even_odd: bool = False


def _opacity(decl):
    return float(decl.get('fill-opacity', 1.0)) * float(decl.get('opacity', 1.0))


def _resolve(element, transform, fill, defs):
    """The element's resolved style (parse_svg.py:288-387): its class rule
    overridden by its attributes (the presentation), then its style
    attribute, each with pydiffvg's rules."""
    presentation = dict(defs[element.attrib['class']]) if 'class' in element.attrib else {}
    presentation.update(element.attrib)
    r = _Resolved(transform, fill, half_width=torch.tensor(0.5))
    if 'transform' in presentation:
        r.transform = transform @ parse_transform(presentation['transform'])
    # presentation: the fill's alpha becomes the product of the opacities
    # given (1 when none is), written into the fill tensor itself
    if 'fill' in presentation:
        r.fill = parse_color(presentation['fill'], defs)
    if isinstance(r.fill, torch.Tensor):
        r.fill[3] = _opacity(presentation)
    if 'fill-rule' in presentation:
        r.even_odd = _even_odd(presentation['fill-rule'], r.even_odd)
    if 'stroke' in presentation:
        r.stroke = parse_color(presentation['stroke'], defs)
    if 'stroke-width' in presentation:
        r.half_width = _half_width(presentation['stroke-width'])
    if 'stroke-opacity' in presentation:
        r.stroke[3] = torch.tensor(float(presentation['stroke-opacity']))
    if 'style' not in presentation:
        return r
    # inline style: its own opacities replace the fill's alpha again; stroke
    # opacity and width count only together with a stroke
    inline = parse_style(presentation['style'], defs)
    if 'fill' in inline:
        r.fill = parse_color(inline['fill'], defs)
    if 'fill-rule' in inline:
        r.even_odd = _even_odd(inline['fill-rule'], r.even_odd)
    if isinstance(r.fill, torch.Tensor):
        r.fill[3] = _opacity(inline)
    if 'stroke' in inline:
        r.stroke = parse_color(inline['stroke'], defs)
        if isinstance(r.stroke, torch.Tensor):
            if 'stroke-opacity' in inline:
                r.stroke[3] = float(inline['stroke-opacity'])
            if 'opacity' in inline:
                r.stroke[3] *= float(inline['opacity'])
        if 'stroke-width' in inline:
            r.half_width = _half_width(inline['stroke-width'])
    for paint in (r.fill, r.stroke):
        if isinstance(paint, LinearGradient):
            paint.begin = _apply(r.transform, paint.begin)
            paint.end = _apply(r.transform, paint.end)
    return r


# --------------------------------------------------------------------------
# shape emission

def _numbers(text):
    return [float(v) for v in re.split(r'[\s,]+', text.strip()) if v]


def _emit(element, style, shapes, groups):
    """Appends the element's shapes and one group for them
    (parse_svg.py:392-516).  Path points are mapped to the canvas and their
    group keeps the identity transform; the other shapes keep their own
    coordinates under the group's transform."""
    tag = _tag(element)
    a = element.attrib
    name = a.get('id', '')
    closed = style.fill is not None
    group_id, with_transform = '', True
    if tag == 'path':
        new = from_svg_path(a['d'], style.transform, closed)
        for k, p in enumerate(new):
            p.source_id = name
            p.id = '{}-{}'.format(name, k) if len(new) > 1 else name
        group_id, with_transform = name, False
    elif tag == 'polygon':
        new = [Polygon(torch.tensor(_numbers(a['points']), dtype=torch.float32).view(-1, 2), closed)]
        group_id = name
    elif tag == 'line':
        ends = [[float(a['x1']), float(a['y1'])], [float(a['x2']), float(a['y2'])]]
        new = [Polygon(torch.tensor(ends), False)]
    elif tag == 'circle':
        new = [Circle(radius=torch.tensor(float(a['r'])), center=torch.tensor([float(a['cx']), float(a['cy'])]))]
    else:  # rect
        w, h = float(a['width']), float(a['height'])
        new = [Rect(p_min=torch.tensor([0.0, 0.0]), p_max=torch.tensor([w, h]))]
    for s in new:
        s.stroke_width = style.half_width
    ids = torch.tensor(list(range(len(shapes), len(shapes) + len(new))))
    shapes.extend(new)
    kw = dict(shape_ids=ids, fill_color=style.fill, stroke_color=style.stroke, use_even_odd_rule=style.even_odd,
              id=group_id)
    if with_transform:
        kw['shape_to_canvas'] = style.transform
    groups.append(ShapeGroup(**kw))


def _walk(element, transform, fill, defs, shapes, groups, top_level):
    """Shapes and groups under `element` in document order.  Definitions are
    read at the top level and in <defs>; a <g> passes down only its
    transform and fill attributes."""
    for child in element:
        tag = _tag(child)
        if tag in _SHAPE_TAGS:
            _emit(child, _resolve(child, transform, fill, defs), shapes, groups)
        elif tag == 'g':
            t = transform @ parse_transform(child.attrib['transform']) if 'transform' in child.attrib else transform
            f = parse_color(child.attrib['fill'], defs) if 'fill' in child.attrib else fill
            _walk(child, t, f, defs, shapes, groups, False)
        elif top_level and tag == 'defs':
            for d in child:
                _register(d, defs)
        elif top_level:
            _register(child, defs)


def parse_scene(node):
    """The root <svg> element as (canvas_width, canvas_height, shapes,
    shape_groups) (parse_svg.py:533-572)."""
    width = height = -1
    if 'viewBox' in node.attrib:
        box = node.attrib['viewBox'].split()
        width, height = _length(box[2]), _length(box[3])
    else:
        for key in ('width', 'height'):
            if key in node.attrib:
                value = _length(node.attrib[key])
                width, height = (value, height) if key == 'width' else (width, value)
            else:
                warnings.warn("Can't find canvas {}.".format(key))
    shapes, groups = [], []
    _walk(node, torch.eye(3), torch.tensor([0.0, 0.0, 0.0, 1.0]), {}, shapes, groups, True)
    return width, height, shapes, groups


def svg_to_scene(filename):
    """Load an SVG file as (canvas_width, canvas_height, shapes, shape_groups)."""
    return parse_scene(etree.parse(filename).getroot())
