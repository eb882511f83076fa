"""SVG path data (the "d" attribute) to segments.

Follows the path data grammar of the SVG 1.1 specification (section 8.3):
commands M/m, L/l, H/h, V/v, C/c, S/s, Q/q, T/t, A/a and Z/z, implicit
repetition of a command's argument groups (a moveto's extra pairs are
linetos), relative coordinates, and the reflected first control point of
S and T.  Elliptical arcs are converted to their centre parameterisation as
in the specification's implementation notes (F.6.5, with radii that are too
small scaled up as in F.6.6); an arc with a zero radius is a line and an
arc whose end points coincide is omitted.  Points are complex numbers
(x + iy).

pydiffvg reads path data through svgpathtools (shape.py:63-159); this module
stands in for that dependency with the same segment model: a flat list of
segments, split into continuous subpaths where one segment does not start
where the previous one ended.
"""
import math

__all__ = ['Line', 'QuadraticBezier', 'CubicBezier', 'Arc', 'parse_path', 'continuous_subpaths']


class Line:
    def __init__(self, start, end):
        self.start, self.end = start, end

    def length(self):
        return abs(self.end - self.start)


class QuadraticBezier:
    def __init__(self, start, control, end):
        self.start, self.control, self.end = start, control, end


class CubicBezier:
    def __init__(self, start, control1, control2, end):
        self.start, self.control1, self.control2, self.end = start, control1, control2, end


class Arc:
    """Elliptical arc with its centre parameterisation: radius = rx + i ry
    (after scaling), phi = x-axis rotation in degrees, theta = start angle
    and delta = swept angle, both in degrees."""

    def __init__(self, start, radius, rotation, large_arc, sweep, end):
        self.start, self.end = start, end
        self.phi = float(rotation)
        self.large_arc, self.sweep = bool(large_arc), bool(sweep)
        rx, ry = abs(radius.real), abs(radius.imag)
        cphi, sphi = math.cos(math.radians(self.phi)), math.sin(math.radians(self.phi))
        dx, dy = (start.real - end.real) / 2.0, (start.imag - end.imag) / 2.0
        x1 = cphi * dx + sphi * dy
        y1 = -sphi * dx + cphi * dy
        lam = (x1 * x1) / (rx * rx) + (y1 * y1) / (ry * ry)
        if lam > 1.0:
            s = math.sqrt(lam)
            rx, ry = rx * s, ry * s
        num = rx * rx * ry * ry - rx * rx * y1 * y1 - ry * ry * x1 * x1
        den = rx * rx * y1 * y1 + ry * ry * x1 * x1
        coef = math.sqrt(max(num, 0.0) / den) if den > 0 else 0.0
        if self.large_arc == self.sweep:
            coef = -coef
        cxp = coef * rx * y1 / ry
        cyp = -coef * ry * x1 / rx
        cx = cphi * cxp - sphi * cyp + (start.real + end.real) / 2.0
        cy = sphi * cxp + cphi * cyp + (start.imag + end.imag) / 2.0
        self.radius = complex(rx, ry)
        self.center = complex(cx, cy)
        ux, uy = (x1 - cxp) / rx, (y1 - cyp) / ry
        vx, vy = (-x1 - cxp) / rx, (-y1 - cyp) / ry
        self.theta = math.degrees(math.atan2(uy, ux))
        delta = math.degrees(math.atan2(ux * vy - uy * vx, ux * vx + uy * vy))
        if not self.sweep and delta > 0:
            delta -= 360.0
        elif self.sweep and delta < 0:
            delta += 360.0
        self.delta = delta


class _Scanner:
    """Numbers, flags and command letters of a path data string."""

    COMMANDS = set('MmZzLlHhVvCcSsQqTtAa')

    def __init__(self, s):
        self.s = s
        self.i = 0
        self.n = len(s)

    def _skip(self):
        while self.i < self.n and (self.s[self.i].isspace() or self.s[self.i] == ','):
            self.i += 1

    def at_end(self):
        self._skip()
        return self.i >= self.n

    def peek_command(self):
        self._skip()
        if self.i < self.n and self.s[self.i] in self.COMMANDS:
            return self.s[self.i]
        return None

    def command(self):
        c = self.peek_command()
        if c is None:
            raise ValueError('path data: expected a command at offset %d in %r' % (self.i, self.s))
        self.i += 1
        return c

    def number(self):
        self._skip()
        s, i, n = self.s, self.i, self.n
        j = i
        if j < n and s[j] in '+-':
            j += 1
        digits = False
        while j < n and s[j].isdigit():
            j += 1
            digits = True
        if j < n and s[j] == '.':
            j += 1
            while j < n and s[j].isdigit():
                j += 1
                digits = True
        if not digits:
            raise ValueError('path data: expected a number at offset %d in %r' % (i, s))
        if j < n and s[j] in 'eE':
            k = j + 1
            if k < n and s[k] in '+-':
                k += 1
            if k < n and s[k].isdigit():
                while k < n and s[k].isdigit():
                    k += 1
                j = k
        self.i = j
        return float(s[i:j])

    def flag(self):
        """An arc flag: a single 0 or 1 (flags may be written without separators)."""
        self._skip()
        if self.i < self.n and self.s[self.i] in '01':
            self.i += 1
            return self.s[self.i - 1] == '1'
        raise ValueError('path data: expected an arc flag at offset %d in %r' % (self.i, self.s))


def parse_path(d):
    """Segments of a path data string, in order."""
    sc = _Scanner(d)
    segments = []
    cur = start = 0j
    cmd = None
    last_cubic_ctrl = last_quad_ctrl = None  # for S / T
    while not sc.at_end():
        c = sc.peek_command()
        if c is not None:
            if cmd is None and c not in 'Mm':
                raise ValueError('path data must begin with a moveto: %r' % d)
            cmd = sc.command()
        elif cmd is None:
            raise ValueError('path data must begin with a moveto: %r' % d)
        elif cmd in 'Mm':
            cmd = 'L' if cmd == 'M' else 'l'  # extra coordinate pairs of a moveto are linetos
        rel = cmd.islower()
        op = cmd.upper()
        if op == 'Z':
            if cur != start:
                segments.append(Line(cur, start))
            cur = start
            last_cubic_ctrl = last_quad_ctrl = None
            continue
        if op == 'M':
            p = complex(sc.number(), sc.number())
            cur = cur + p if rel else p
            start = cur
            last_cubic_ctrl = last_quad_ctrl = None
            continue
        cubic_ctrl = quad_ctrl = None
        if op == 'L':
            p = complex(sc.number(), sc.number())
            end = cur + p if rel else p
            segments.append(Line(cur, end))
        elif op == 'H':
            x = sc.number()
            end = complex(cur.real + x if rel else x, cur.imag)
            segments.append(Line(cur, end))
        elif op == 'V':
            y = sc.number()
            end = complex(cur.real, cur.imag + y if rel else y)
            segments.append(Line(cur, end))
        elif op == 'C':
            c1 = complex(sc.number(), sc.number())
            c2 = complex(sc.number(), sc.number())
            end = complex(sc.number(), sc.number())
            if rel:
                c1, c2, end = cur + c1, cur + c2, cur + end
            segments.append(CubicBezier(cur, c1, c2, end))
            cubic_ctrl = c2
        elif op == 'S':
            c2 = complex(sc.number(), sc.number())
            end = complex(sc.number(), sc.number())
            if rel:
                c2, end = cur + c2, cur + end
            c1 = 2 * cur - last_cubic_ctrl if last_cubic_ctrl is not None else cur
            segments.append(CubicBezier(cur, c1, c2, end))
            cubic_ctrl = c2
        elif op == 'Q':
            c1 = complex(sc.number(), sc.number())
            end = complex(sc.number(), sc.number())
            if rel:
                c1, end = cur + c1, cur + end
            segments.append(QuadraticBezier(cur, c1, end))
            quad_ctrl = c1
        elif op == 'T':
            end = complex(sc.number(), sc.number())
            if rel:
                end = cur + end
            c1 = 2 * cur - last_quad_ctrl if last_quad_ctrl is not None else cur
            segments.append(QuadraticBezier(cur, c1, end))
            quad_ctrl = c1
        elif op == 'A':
            rx, ry = sc.number(), sc.number()
            rot = sc.number()
            large, sweep = sc.flag(), sc.flag()
            end = complex(sc.number(), sc.number())
            if rel:
                end = cur + end
            if end != cur:
                if rx == 0 or ry == 0:
                    segments.append(Line(cur, end))
                else:
                    segments.append(Arc(cur, complex(rx, ry), rot, large, sweep, end))
        cur = end
        last_cubic_ctrl, last_quad_ctrl = cubic_ctrl, quad_ctrl
    return segments


def continuous_subpaths(segments):
    """Split a segment list where a segment does not start at the previous end."""
    subpaths = []
    for seg in segments:
        if subpaths and subpaths[-1][-1].end == seg.start:
            subpaths[-1].append(seg)
        else:
            subpaths.append([seg])
    return subpaths
