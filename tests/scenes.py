"""z2d spec scenes restated against a fill/composite backend.

Each function below re-expresses the drawing commands of one of z2d's spec
scenes (spec/NNN_*.zig, 0BSD) that exercise only painter.fill and the
compositor, using a small stand-in for z2d's Context (src/Context.zig:36-61,
592-607, 679-699).  A backend provides fill(surface, pattern, nodes, opts)
and composite(dst, x, y, ops, precision): the oracle for golden pinning, the
GPU library for parity.
"""
from __future__ import annotations

import math
from fractions import Fraction

from z2d_gb300 import abi
from z2d_gb300.path import Path, tf_distance, tf_inverse, tf_mul, tf_rotate, tf_scale, tf_translate
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, FillOptions, Gradient, Operation, Pattern, Pixel, wrap_dither


class Ctx:
    """The subset of z2d.Context the fill scenes use."""

    def __init__(self, backend, surface: Surface):
        self.backend = backend
        self.surface = surface
        self.pattern = Pattern.from_pixel(Pixel.rgba(0, 0, 0, 0xFF))
        self.aa = "default"
        self.fill_rule = "non_zero"
        self.operator = "src_over"
        self.precision = "integer"
        self.tolerance = 0.1
        self.dither = "none"
        self.transformation = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
        self.line_width = 2.0      # Context defaults (src/Context.zig:36-61)
        self.line_join = "miter"
        self.line_cap = "butt"
        self.miter_limit = 10.0
        self.dashes = ()
        self.dash_offset = 0.0
        self.hairline = False
        self.path = Path()

    # the CTM (src/Context.zig:340-380): the path transforms points with it
    def set_transformation(self, t):
        self.transformation = tuple(float(v) for v in t)
        self.path.transformation = self.transformation

    def get_transformation(self):
        return self.transformation

    def set_identity(self):
        self.set_transformation((1.0, 0.0, 0.0, 1.0, 0.0, 0.0))

    def translate(self, tx, ty):
        self.set_transformation(tf_translate(self.transformation, tx, ty))

    def scale(self, sx, sy):
        self.set_transformation(tf_scale(self.transformation, sx, sy))

    def rotate(self, angle):
        self.set_transformation(tf_rotate(self.transformation, angle))

    def set_source_pattern(self, pattern):
        """Context.setSource (src/Context.zig:115-121): a gradient takes the
        current transformation."""
        if pattern.kind == abi.PATTERN_GRADIENT:
            try:
                pattern.gradient.set_transformation(self.transformation)
            except ValueError:
                return
        self.pattern = pattern

    def mul(self, m):
        self.set_transformation(tf_mul(self.transformation, m))

    def device_to_user_distance(self, x, y):
        return tf_distance(tf_inverse(self.transformation), x, y)

    def set_tolerance(self, t):  # Context.setTolerance (src/Context.zig:303-307)
        self.tolerance = max(float(t), 0.001)
        self.path.tolerance = self.tolerance

    def arc(self, xc, yc, r, a1, a2):
        self.path.arc(xc, yc, r, a1, a2)

    def arc_negative(self, xc, yc, r, a1, a2):
        self.path.arc_negative(xc, yc, r, a1, a2)

    def set_source(self, px: Pixel):
        self.pattern = Pattern.from_pixel(px)

    def move_to(self, x, y):
        self.path.move_to(x, y)

    def line_to(self, x, y):
        self.path.line_to(x, y)

    def curve_to(self, *a):
        self.path.curve_to(*a)

    def close_path(self):
        self.path.close()

    def reset_path(self):
        self.path.reset()

    def stroke(self):
        from z2d_gb300.types import StrokeOptions
        pat = wrap_dither(self.pattern, self.dither, self.surface.format)
        opts = StrokeOptions(anti_aliasing=self.aa, line_cap=self.line_cap, line_join=self.line_join,
                             line_width=self.line_width, miter_limit=self.miter_limit, operator=self.operator,
                             precision=self.precision, tolerance=self.tolerance,
                             transformation=self.transformation, dashes=self.dashes,
                             dash_offset=self.dash_offset, hairline=self.hairline)
        rc = self.backend.stroke(self.surface, pat, self.path.nodes, opts)
        if rc != abi.OK:
            raise RuntimeError(f"stroke failed: {rc}")

    def fill(self):
        pat = wrap_dither(self.pattern, self.dither, self.surface.format)
        opts = FillOptions(self.aa, self.fill_rule, self.operator, self.precision, self.tolerance)
        rc = self.backend.fill(self.surface, pat, self.path.nodes, opts)
        if rc != abi.OK:
            raise RuntimeError(f"fill failed: {rc}")


def _white_rgb():
    return Pixel.rgb(0xFF, 0xFF, 0xFF)


# --------------------------------------------------------------- fill scenes
def s003_fill_triangle(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    m = 10
    c.move_to(0 + m, 0 + m)
    c.line_to(w - m - 1, 0 + m)
    c.line_to(w // 2 - 1, h - m - 1)
    c.close_path()
    c.fill()
    return s


def s004_fill_square(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    m = 50
    c.move_to(m, m)
    c.line_to(w - m - 1, m)
    c.line_to(w - m - 1, h - m - 1)
    c.line_to(m, h - m - 1)
    c.close_path()
    c.fill()
    return s


def s005_fill_trapezoid(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    mt, mb, my = 89, 50, 100
    c.move_to(mt, my)
    c.line_to(w - mt - 1, my)
    c.line_to(w - mb - 1, h - my - 1)
    c.line_to(mb, h - my - 1)
    c.close_path()
    c.fill()
    return s


def _star(c, w, h, margin, xs, ys, xo=0, yo=0, sw=None, sh=None):
    sw = w if sw is None else sw
    sh = h if sh is None else sh
    c.move_to(xo + sw // 2, yo + margin)
    c.line_to(xo + sw - margin * xs - 1, yo + sh - margin - 1)
    c.line_to(xo + margin, yo + margin * ys)
    c.line_to(xo + sw - margin - 1, yo + margin * ys)
    c.line_to(xo + margin * xs, yo + sh - margin - 1)
    c.close_path()


def s006_fill_star_even_odd(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.fill_rule = "even_odd"
    _star(c, w, h, 20, 3, 5)
    c.fill()
    return s


def s016_fill_star_non_zero(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.fill_rule = "non_zero"
    _star(c, w, h, 20, 3, 5)
    c.fill()
    return s


def s007_fill_bezier(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.move_to(19, 249)
    c.curve_to(89, 49, 209, 49, 279, 249)
    c.close_path()
    c.fill()
    return s


def s013_fill_combined(be, aa):
    w, h = 600, 400
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    scw, sch = w // 3, h // 2
    m = 10
    c.move_to(m, m)
    c.line_to(scw - m - 1, m)
    c.line_to(scw // 2 - 1, sch - m - 1)
    c.close_path()
    m = 50
    xo = scw
    c.move_to(xo + m, m)
    c.line_to(xo + scw - m - 1, m)
    c.line_to(xo + scw - m - 1, sch - m - 1)
    c.line_to(xo + m, sch - m - 1)
    c.close_path()
    tmt, tmb, tmy = 59, 33, 66
    xo = scw * 2
    c.move_to(xo + tmt, tmy)
    c.line_to(xo + scw - tmt - 1, tmy)
    c.line_to(xo + scw - tmb - 1, sch - tmy - 1)
    c.line_to(xo + tmb, sch - tmy - 1)
    c.close_path()
    m = 13
    xo = w // 6
    yo = sch
    _star(c, w, h, m, 3, 5, xo, yo, scw, sch)
    xo += scw
    c.move_to(xo + 12, yo + 166)
    c.curve_to(xo + 59, yo + 32, xo + 139, yo + 32, xo + 186, yo + 166)
    c.close_path()
    c.fill()
    return s


def _tri(c, w, h, m=10):
    c.move_to(m, m)
    c.line_to(w - m - 1, m)
    c.line_to(w // 2 - 1, h - m - 1)
    c.close_path()


def s024_fill_triangle_direct_cross_format(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(Pixel.rgba(0xFF, 0x8A, 0xA5, 0xFF))
    c.aa = aa
    _tri(c, 300, 300)
    c.fill()
    return s


def s025_fill_diamond_clipped(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.move_to(w // 2, 0 - h // 10)
    c.line_to(w + w // 10, h // 2)
    c.line_to(w // 2, h + h // 10)
    c.line_to(0 - w // 10, h // 2)
    c.close_path()
    c.fill()
    return s


def s026_fill_triangle_full(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.move_to(0, 0)
    c.line_to(w, 0)
    c.line_to(w // 2, h)
    c.close_path()
    c.fill()
    return s


def s028_fill_bezier_tolerance(be, aa):
    s = Surface.init("rgb", 900, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    for x0, tol in ((0, None), (300, 3), (600, 10)):
        if tol is not None:
            c.tolerance = tol
        c.reset_path()
        c.move_to(x0 + 19, 224)
        c.curve_to(x0 + 89, 49, x0 + 209, 49, x0 + 279, 224)
        c.close_path()
        c.fill()
    return s


def s031_fill_quad_bezier(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.move_to(20, 130)
    c.curve_to(20, 130, 20, 20, 130, 20)
    c.close_path()
    c.move_to(170, 20)
    c.curve_to(280, 20, 280, 20, 280, 130)
    c.close_path()
    c.move_to(280, 170)
    c.curve_to(280, 280, 170, 280, 170, 280)
    c.close_path()
    c.move_to(130, 280)
    c.curve_to(20, 280, 20, 280, 20, 170)
    c.close_path()
    c.fill()
    return s


def s046_fill_triangle_alpha(be, aa):
    s = Surface.init_pixel(Pixel.rgb(0xFF, 0xFF, 0xFF), 300, 300)
    c = Ctx(be, s)
    c.set_source(Pixel.alpha8(255))
    c.aa = aa
    _tri(c, 300, 300)
    c.fill()
    return s


def _alpha_tri(fmt, px):
    def scene(be, aa):
        s = Surface.init(fmt, 300, 300)
        c = Ctx(be, s)
        c.set_source(px)
        c.aa = aa
        _tri(c, 300, 300)
        c.fill()
        return s
    return scene


def s048_fill_triangle_static(be, aa):
    s = Surface.init("rgb", 300, 300)
    p = Path()
    _tri_path(p)
    rc = be.fill(s, Pattern.from_pixel(_white_rgb()), p.nodes, FillOptions(anti_aliasing=aa))
    assert rc == abi.OK
    return s


def _tri_path(p, w=300, h=300, m=10):
    p.move_to(m, m)
    p.line_to(w - m - 1, m)
    p.line_to(w // 2 - 1, h - m - 1)
    p.close()


def s079_fill_degenerate_lineto(be, aa):
    s = Surface.init("rgb", 100, 200)
    c = Ctx(be, s)
    c.aa = aa
    c.set_source(_white_rgb())
    groups = [
        [("m", 180, 180), ("l", 190, 190), ("c",)],
        [("m", 10, 10), ("l", 20, 10), ("l", 20, 20), ("l", 10, 20), ("c",), ("m", 50, 10), ("l", 70, 20), ("c",)],
        [("m", 10, 50), ("l", 30, 70), ("c",), ("m", 50, 50), ("l", 60, 50), ("l", 60, 60), ("l", 50, 60), ("c",)],
        [("m", -30, 80), ("l", -10, 100), ("c",), ("m", 50, 80), ("l", 60, 80), ("l", 60, 90), ("l", 50, 90), ("c",)],
        [("m", 10, 110), ("l", 30, 130), ("c",), ("m", 150, 110), ("l", 160, 110), ("l", 160, 120), ("l", 150, 120),
         ("c",)],
        [("m", 10, 140), ("l", 20, 140), ("l", 20, 150), ("l", 10, 150), ("c",), ("m", 50, 140), ("l", 70, 150), ("c",)],
    ]
    for g in groups:
        c.reset_path()
        for cmd in g:
            if cmd[0] == "m":
                c.move_to(cmd[1], cmd[2])
            elif cmd[0] == "l":
                c.line_to(cmd[1], cmd[2])
            else:
                c.close_path()
        c.fill()
    return s


# --------------------------------------------------------- gradient scenes
def _linear_draw(be, dst, scratch, sx, sy, x0, y0, x1, y1):
    # spec/061_linear_gradient.zig draw()
    g = Gradient.linear(x0, y0, x1, y1)
    g.add_stop(0, Color.rgb(1, 0, 0))
    g.add_stop(0.5, Color.rgb(0, 1, 0))
    g.add_stop(1, Color.rgb(0, 0, 1))
    assert be.composite(scratch, 0, 0, [Operation("src_over", src=Pattern.from_gradient(g))]) == abi.OK
    assert be.composite(dst, sx, sy, [Operation("src_over", src=scratch)]) == abi.OK


def s061_linear_gradient(be, aa=None):
    dst = Surface.init("rgb", 200, 400)
    scratch = Surface.init("rgb", 100, 100)
    for args in ((0, 0, 0, 49, 99, 49), (100, 0, 99, 49, 0, 49), (0, 100, 49, 0, 49, 99),
                 (100, 100, 49, 99, 49, 0), (0, 200, 0, 0, 99, 99), (100, 200, 99, 0, 0, 99),
                 (0, 300, 0, 99, 99, 0), (100, 300, 99, 99, 0, 0)):
        _linear_draw(be, dst, scratch, *args)
    return dst


def _gradient_draw(be, dst, scratch, sx, sy, g):
    assert be.composite(scratch, 0, 0, [Operation("src_over", src=Pattern.from_gradient(g))]) == abi.OK
    assert be.composite(dst, sx, sy, [Operation("src_over", src=scratch)]) == abi.OK


def s062_hsl_gradient(be, aa=None):
    dst = Surface.init("rgb", 100, 200)
    for w, h, sx, sy, x0, y0, x1, y1, c0, c1 in (
        (100, 100, 0, 0, 0, 49, 99, 49, Color.hsl(300, 1, 0.5), Color.hsl(60, 1, 0.5)),
        (50, 100, 0, 100, 0, 49, 49, 49, Color.hsl(0, 1, 0.5), Color.hsl(0, 0, 0.5)),
        (50, 100, 50, 100, 49, 49, 0, 49, Color.hsl(180, 1, 0.5), Color.hsl(180, 0, 0.5)),
        (100, 50, 0, 100, 49, 0, 49, 49, Color.hsl(0, 0, 1, 1), Color.hsl(0, 0, 0.5, 0)),
        (100, 50, 0, 150, 49, 49, 49, 0, Color.hsl(0, 0, 0, 1), Color.hsl(0, 0, 0.5, 0)),
    ):
        g = Gradient.linear(x0, y0, x1, y1, method="hsl", polar="shorter")
        g.add_stop(0, c0)
        g.add_stop(1, c1)
        _gradient_draw(be, dst, Surface.init("rgba", w, h), sx, sy, g)
    return dst


def s063_radial_gradient(be, aa=None):
    dst = Surface.init("rgba", 300, 500)
    cases = [(100 * x, 100 * y, 49 + 25 * (float(x) - 1), 49 + 25 * (float(y) - 1), 5, 49, 49, 50)
             for y in range(3) for x in range(3)]
    cases += [(0, 300, 49, 49, 0, 49, 49, 50), (100, 300, 49, 49, 50, 49, 49, 0), (200, 300, 49, 49, 50, 49, 49, 50),
              (0, 400, 49, 49, 0, 49, 49, 0), (100, 400, 10, 49, 0, 49, 49, 25), (200, 400, 49, 49, 49, 49, 49, 50)]
    for sx, sy, ix, iy, ir, ox, oy, orad in cases:
        g = Gradient.radial(ix, iy, ir, ox, oy, orad)
        g.add_stop(0, Color.rgb(1, 0, 0))
        g.add_stop(0.5, Color.rgb(0, 1, 0))
        g.add_stop(1, Color.rgb(0, 0, 1))
        _gradient_draw(be, dst, Surface.init("rgba", 100, 100), sx, sy, g)
    return dst


def _rgb_stops(g):
    g.add_stop(0, Color.rgb(1, 0, 0))
    g.add_stop(0.5, Color.rgb(0, 1, 0))
    g.add_stop(1, Color.rgb(0, 0, 1))
    return g


def s064_radial_source(be, aa):
    s = Surface.init("rgb", 100, 100)
    c = Ctx(be, s)
    c.aa = aa
    c.pattern = Pattern.from_gradient(_rgb_stops(Gradient.radial(49, 49, 0, 49, 49, 50)))
    _poly(c, [(0, 0), (100, 0), (100, 100), (0, 100)])
    c.fill()
    return s


def s065_conic_gradient(be, aa=None):
    dst = Surface.init("rgba", 200, 200)
    for y in range(2):
        for x in range(2):
            g = Gradient.conic(49, 49, math.pi / 2.0 * float(y * 2 + x), method="hsl", polar="increasing")
            g.add_stop(0, Color.hsl(0, 1, 0.5))
            g.add_stop(1, Color.hsl(360, 1, 0.5))
            _gradient_draw(be, dst, Surface.init("rgba", 100, 100), 100 * x, 100 * y, g)
    return dst


def s066_conic_pie_gradient(be, aa):
    s = Surface.init("rgb", 300, 300)
    g = Gradient.conic(149, 149, 0)
    third, two_thirds = Fraction(1, 3), Fraction(2, 3)
    g.add_stop(0, Color.rgb(1, 0, 0))
    g.add_stop(float(third), Color.rgb(1, 0, 0))
    g.add_stop(float(third + Fraction("0.005")), Color.rgb(0, 1, 0))
    g.add_stop(float(two_thirds), Color.rgb(0, 1, 0))
    g.add_stop(float(two_thirds + Fraction("0.005")), Color.rgb(0, 0, 1))
    g.add_stop(1, Color.rgb(0, 0, 1))
    c = Ctx(be, s)
    c.aa = aa
    c.pattern = Pattern.from_gradient(g)
    c.arc(149, 149, 100, 0, math.pi * 2)
    c.close_path()
    c.fill()
    return s


def _f32(fr: Fraction) -> float:
    """The f32 nearest to an exact value (Zig rounds compile-time constants
    once; a double in between could round twice)."""
    import numpy as np
    c = np.float32(float(fr))
    best = c
    for cand in (np.nextafter(c, np.float32(-np.inf)), np.nextafter(c, np.float32(np.inf))):
        if abs(Fraction(float(cand)) - fr) < abs(Fraction(float(best)) - fr):
            best = cand
    return float(best)


def _unit_square(c, size):
    _poly(c, [(0, 0), (size, 0), (size, size), (0, size)])


def s067_gradient_transforms(be, aa):
    s = Surface.init("rgb", 200, 200)
    c = Ctx(be, s)
    c.scale(2, 2)
    c.aa = aa
    c.set_source_pattern(Pattern.from_gradient(_rgb_stops(Gradient.linear(0, 0, 50, 50))))
    _unit_square(c, 50)
    c.fill()
    radial = _rgb_stops(Gradient.radial(25, 50, 0, 25, 50, 50))
    c.set_identity()
    c.mul((1.0, 0.5, 0.0, 1.0, 0.0, 0.0))  # skew: by = 0.5
    c.translate(100, 0)
    c.set_source_pattern(Pattern.from_gradient(radial))
    c.set_identity()
    c.translate(100, 0)
    c.reset_path()
    _unit_square(c, 100)
    c.fill()
    conic = Gradient.conic(50, 50, 0, method="hsl", polar="increasing")
    conic.add_stop(0, Color.hsl(0, 1, 0.5))
    conic.add_stop(1, Color.hsl(360, 1, 0.5))
    c.set_identity()
    c.scale(2, 1)
    c.translate(0, 100)
    c.set_source_pattern(Pattern.from_gradient(conic))
    c.reset_path()
    _unit_square(c, 100)
    c.fill()
    return s


def s068_gradient_deband(be, aa=None):
    dst = Surface.init_pixel(Pixel.rgb(255, 255, 255), 500, 500)
    for sy, gray, bits, dither in ((0, False, 8, "none"), (100, False, 8, "bayer"), (200, True, 8, "none"),
                                   (300, True, 4, "none"), (400, True, 4, "bayer")):
        fmt = ("alpha4" if bits == 4 else "alpha8") if gray else "rgb"
        scratch = Surface.init(fmt, 500, 100)
        g = Gradient.linear(0, 50, 500, 50)
        if gray:
            g.add_stop(0, Color.rgb(1, 1, 1, 0))
            g.add_stop(1, Color.rgb(0, 0, 0, 1))
        else:
            g.add_stop(0, Color.rgb(*(_f32(Fraction(v, 255)) for v in (27, 93, 124))))
            g.add_stop(1, Color.rgb(*(_f32(Fraction(v, 255)) for v in (38, 32, 16))))
        assert be.composite(scratch, 0, 0, [Operation("src_over", src=Pattern.dither(dither, g, bits))]) == abi.OK
        assert be.composite(dst, 0, sy, [Operation("src_over", src=scratch)]) == abi.OK
    return dst


def s069_gradient_dither_context(be, aa):
    s = Surface.init("alpha4", 400, 150)
    g = Gradient.linear(0, 25, 400, 25)
    g.add_stop(0, Color.rgb(0, 0, 0, 0))
    g.add_stop(1, Color.rgb(1, 1, 1, 1))
    c = Ctx(be, s)
    c.aa = aa
    for ty, dither in ((None, "none"), (50, "bayer"), (100, "blue_noise")):
        if ty is not None:
            c.reset_path()
            c.set_identity()
            c.translate(0, ty)
        c.set_source_pattern(Pattern.from_gradient(g))
        c.dither = dither
        _poly(c, [(0, 0), (400, 0), (400, 50), (0, 50)])
        c.fill()
    return s


def s070_compositor_ops(be, aa):
    s = Surface.init_pixel(Pixel.rgb(255, 255, 255), 460, 3090)
    for i, op in enumerate(abi.OPERATORS):
        for j in range(4):
            transparent = (j % 2) == 1
            bg = Pixel.from_color(Color.rgb(0.69, 0.23, 0.21, 0.9) if transparent else Color.rgb(0.69, 0.23, 0.21))
            fg = Pixel.from_color(Color.rgb(0.56, 0.50, 0.89, 0.8) if transparent else Color.rgb(0.56, 0.50, 0.89))
            scratch = Surface.init("rgba", 100, 100)
            c = Ctx(be, scratch)
            c.aa = aa
            c.precision = "integer" if j < 2 else "float"
            c.set_source(bg)
            _poly(c, [(0, 0), (75, 0), (75, 75), (0, 75)])
            c.fill()
            c.set_source(fg)
            c.operator = op
            c.reset_path()
            c.translate(25, 25)
            _poly(c, [(0, 0), (75, 0), (75, 75), (0, 75)])
            c.fill()
            assert be.composite(s, 10 + 110 * j, 10 + 110 * i, [Operation("src_over", src=scratch)]) == abi.OK
    return s


def s059_stroke_star_gradient(be, aa):
    w = h = 300
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.aa = aa
    c.line_width = 10
    c.line_join = "round"
    m, xs, ys = 20, 3, 5
    c.set_source_pattern(Pattern.from_gradient(_rgb_stops(Gradient.linear(m * 3, h // 2, w - m * 3, h // 2))))
    _poly(c, [(w // 2, m), (w - m * xs - 1, h - m - 1), (m, m * ys), (w - m - 1, m * ys), (m * xs, h - m - 1)])
    c.stroke()
    return s


def _gamma_scene(be, aa=None):
    """spec/071_gamma_linear.zig and 072_gamma_srgb.zig (the same drawing,
    exported with the linear or the sRGB profile)."""
    W, H = 400, 300
    s = Surface.init("rgb", W, H)
    c = Ctx(be, s)
    c.aa = "none"

    def gray(pos, profile):
        col = Color.rgb(0.3, 0.3, 0.3) if profile == "linear" else Color.srgb(0.3, 0.3, 0.3)
        c.set_source(Pixel.from_color(col))
        c.translate(0, pos * H / 2)
        _poly(c, [(0, 0), (W, 0), (W, H // 2), (0, H // 2)])
        c.set_identity()
        c.fill()
        c.reset_path()

    def gradient(pos, stop_profile, method):
        mk = Color.rgb if stop_profile == "linear" else Color.srgb
        off = 30.0
        gw, gh = W - off * 2, (H - off * 2) / 4
        g = Gradient.linear(0, gh / 2, gw, gh / 2, method=method)
        g.add_stop(0, mk(0.80, 0, 0))
        g.add_stop(0.5, mk(0, 0.80, 0))
        g.add_stop(1, mk(0, 0, 0.80))
        c.translate(off, off + gh * pos)
        c.set_source_pattern(Pattern.from_gradient(g))
        _poly(c, [(0, 0), (gw, 0), (gw, gh), (0, gh)])
        c.set_identity()
        c.fill()
        c.reset_path()
        c.set_source(Pixel.rgb(0, 0, 0))

    gray(0, "linear")
    gray(1, "srgb")
    gradient(0, "linear", "linear_rgb")
    gradient(1, "srgb", "linear_rgb")
    gradient(2, "linear", "srgb")
    gradient(3, "srgb", "srgb")
    return s


# scenes whose goldens carry a colour profile: name -> (scene, profile)
EXPORT_SCENES = {
    "071_gamma_linear": (_gamma_scene, "linear"),
    "072_gamma_srgb": (_gamma_scene, "srgb"),
}


# ------------------------------------------------------------- stroke scenes
def _stroke_canvas(be, aa, w, h):
    s = Surface.init("rgb", w, h)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    return s, c


def s008_stroke_triangle(be, aa):
    w = h = 300
    s, c = _stroke_canvas(be, aa, w, h)
    m = 10
    c.move_to(0 + m, 0 + m)
    c.line_to(w - m - 1, 0 + m)
    c.line_to(w // 2 - 1, h - m - 1)
    c.close_path()
    c.stroke()
    return s


def s009_stroke_square(be, aa):
    w = h = 300
    s, c = _stroke_canvas(be, aa, w, h)
    m = 50
    c.move_to(0 + m, 0 + m)
    c.line_to(w - m - 1, 0 + m)
    c.line_to(w - m - 1, h - m - 1)
    c.line_to(0 + m, h - m - 1)
    c.close_path()
    c.stroke()
    return s


def s010_stroke_trapezoid(be, aa):
    w = h = 300
    s, c = _stroke_canvas(be, aa, w, h)
    mt, mb, my = 89, 50, 100
    c.move_to(0 + mt, 0 + my)
    c.line_to(w - mt - 1, 0 + my)
    c.line_to(w - mb - 1, h - my - 1)
    c.line_to(0 + mb, h - my - 1)
    c.close_path()
    c.stroke()
    return s


def _stroke_star(c, w, h):
    m, xs, ys = 20, 3, 5
    c.move_to(w // 2, 0 + m)
    c.line_to(w - m * xs - 1, h - m - 1)
    c.line_to(0 + m, 0 + m * ys)
    c.line_to(w - m - 1, 0 + m * ys)
    c.line_to(0 + m * xs, h - m - 1)
    c.close_path()


def s011_stroke_star(be, aa):
    s, c = _stroke_canvas(be, aa, 300, 300)
    c.line_width = 6
    _stroke_star(c, 300, 300)
    c.stroke()
    return s


def s017_stroke_star_round(be, aa):
    s, c = _stroke_canvas(be, aa, 300, 300)
    c.line_width = 10
    c.line_join = "round"
    _stroke_star(c, 300, 300)
    c.stroke()
    return s


def s012_stroke_bezier(be, aa):
    s, c = _stroke_canvas(be, aa, 300, 300)
    c.move_to(19, 149)
    c.curve_to(89, 0, 209, 0, 279, 149)
    c.stroke()
    c.line_width = 6
    c.reset_path()
    c.move_to(19, 199)
    c.curve_to(89, 24, 209, 24, 279, 199)
    c.stroke()
    c.line_width = 10
    c.reset_path()
    c.move_to(19, 249)
    c.curve_to(89, 49, 209, 49, 279, 249)
    c.stroke()
    return s


def s014_stroke_lines(be, aa):
    w, h = 800, 400
    s, c = _stroke_canvas(be, aa, w, h)
    sw, sh, m = w // 4, h // 2, 10
    x, y = 0, 0
    c.move_to(x + m, y + m)
    c.line_to(x + sw - m - 1, y + sh - m - 1)
    x = sw
    c.move_to(x + m, y + sh - m - 1)
    c.line_to(x + sw - m - 1, y + m)
    x, y = 0, sh
    c.move_to(x + sw - m - 1, y + m)
    c.line_to(x + m, y + sh - m - 1)
    x, y = sw, sh
    c.move_to(x + sw - m - 1, y + sh - m - 1)
    c.line_to(x + m, y + m)
    x, y = sw * 2, 0
    c.move_to(x + m, y + sh // 2)
    c.line_to(x + sw - m - 1, y + sh // 2)
    x, y = sw * 2, sh
    c.move_to(x + sw // 2, y + m)
    c.line_to(x + sw // 2, y + sh - m - 1)
    x, y = sw * 3, 0
    c.move_to(x + sw // 2, y + sh - m - 1)
    c.line_to(x + sw // 2, y + m)
    x, y = sw * 3, sh
    c.move_to(x + sw - m - 1, y + sh // 2)
    c.line_to(x + m, y + sh // 2)
    c.stroke()
    return s


_SPIRAL = [(10, 10), (100, 20), (110, 120), (10, 110), (20, 30), (90, 40), (95, 100), (30, 95), (30, 50), (80, 50),
           (75, 85), (45, 80), (50, 60), (65, 70)]


def _spirals(c):
    xo, yo = 120, 130
    for fx, fy in ((False, False), (True, False), (False, True), (True, True)):
        for i, (px, py) in enumerate(_SPIRAL):
            x = (xo + 120 - px) if fx else px
            y = (yo + 130 - py) if fy else py
            (c.move_to if i == 0 else c.line_to)(x, y)


def s015_stroke_miter(be, aa):
    s, c = _stroke_canvas(be, aa, 240, 260)
    c.line_width = 6
    _spirals(c)
    c.stroke()
    return s


def s018_stroke_square_spiral_round(be, aa):
    s, c = _stroke_canvas(be, aa, 240, 260)
    c.line_width = 10
    c.line_join = "round"
    _spirals(c)
    c.stroke()
    return s


def s019_stroke_bevel_miterlimit(be, aa):
    s, c = _stroke_canvas(be, aa, 375, 560)
    c.line_width = 5
    settings = [("bevel", 10.0), ("miter", 4.0), ("miter", 1.0), ("miter", 6.0), ("miter", 10.0)]
    xs = [(10, 80, 150), (170, 205, 240), (260, 280, 300), (320, 327.5, 335), (355, 360, 365)]
    for row, (join, limit) in enumerate(settings):
        c.line_join = join
        if join == "miter":
            c.miter_limit = limit
        c.reset_path()
        y = 90 + 100 * row
        for x0, x1, x2 in xs:
            c.move_to(x0, y)
            c.line_to(x1, y - 30)
            c.line_to(x2, y)
        c.stroke()
    return s


def _caps(be, aa, cap):
    w, h = 800, 600
    s, c = _stroke_canvas(be, aa, w, h)
    c.line_cap = cap
    if cap == "round":
        c.line_join = "round"
    c.line_width = 20
    sw, m = w // 4, 30
    sh = h / 3
    x, y = 0.0, 0.0
    c.move_to(x + m, y + m)
    c.line_to(x + sw - m - 1, y + sh - m - 1)
    x = sw
    c.move_to(x + m, y + sh - m - 1)
    c.line_to(x + sw - m - 1, y + m)
    x, y = 0, sh
    c.move_to(x + sw - m - 1, y + m)
    c.line_to(x + m, y + sh - m - 1)
    x, y = sw, sh
    c.move_to(x + sw - m - 1, y + sh - m - 1)
    c.line_to(x + m, y + m)
    x, y = sw * 2, 0
    c.move_to(x + m, y + sh / 2)
    c.line_to(x + sw - m - 1, y + sh / 2)
    x, y = sw * 2, sh
    c.move_to(x + sw / 2, y + m)
    c.line_to(x + sw / 2, y + sh - m - 1)
    x, y = sw * 3, 0
    c.move_to(x + sw / 2, y + sh - m - 1)
    c.line_to(x + sw / 2, y + m)
    x, y = sw * 3, sh
    c.move_to(x + sw - m - 1, y + sh / 2)
    c.line_to(x + m, y + sh / 2)
    x, y = 0, sh * 2
    c.move_to(x + m, y + m)
    c.line_to(x + sw - m - 1, y + sh / 2 - 1)
    c.line_to(x + m, y + sh - m - 1)
    x = sw
    c.move_to(x + sw - m - 1, y + m)
    c.line_to(x + m, y + sh / 2 - 1)
    c.line_to(x + sw - m - 1, y + sh - m - 1)
    x = sw * 2
    sh = sh / 2
    c.move_to(x + m, y + m)
    c.line_to(x + sw / 2 - 1, y + sh - m - 1)
    c.line_to(x + sw - m - 1, y + m)
    x = sw * 3
    c.move_to(x + m, y + sh - m - 1)
    c.line_to(x + sw / 2 - 1, y + m)
    c.line_to(x + sw - m - 1, y + sh - m - 1)
    x = sw * 2
    y = y + sh
    c.move_to(x + sw - m - 1, y + sh - m - 1)
    c.line_to(x + sw / 2 - 1, y + m)
    c.line_to(x + m, y + sh - m - 1)
    x = sw * 3
    c.move_to(x + sw - m - 1, y + m)
    c.line_to(x + sw / 2 - 1, y + sh - m - 1)
    c.line_to(x + m, y + m)
    c.stroke()
    c.set_source(Pixel.rgb(0xF3, 0x00, 0x00))
    c.line_width = 1
    c.stroke()
    return s


def s020_stroke_lines_round_caps(be, aa):
    return _caps(be, aa, "round")


def s021_stroke_lines_square_caps(be, aa):
    return _caps(be, aa, "square")


def s022_stroke_lines_butt_caps(be, aa):
    return _caps(be, aa, "butt")


def _lines(c, w, h):
    sw, sh, m = w // 4, h // 2, 10
    c.move_to(m, m)
    c.line_to(sw - m - 1, sh - m - 1)
    c.move_to(sw + m, sh - m - 1)
    c.line_to(sw + sw - m - 1, m)
    c.move_to(sw - m - 1, sh + m)
    c.line_to(m, sh + sh - m - 1)
    c.move_to(sw + sw - m - 1, sh + sh - m - 1)
    c.line_to(sw + m, sh + m)
    c.move_to(sw * 2 + m, sh // 2)
    c.line_to(sw * 2 + sw - m - 1, sh // 2)
    c.move_to(sw * 2 + sw // 2, sh + m)
    c.line_to(sw * 2 + sw // 2, sh + sh - m - 1)
    c.move_to(sw * 3 + sw // 2, sh - m - 1)
    c.line_to(sw * 3 + sw // 2, m)
    c.move_to(sw * 3 + sw - m - 1, sh + sh // 2)
    c.line_to(sw * 3 + m, sh + sh // 2)


def s054_stroke_lines_dashed(be, aa):
    s, c = _stroke_canvas(be, aa, 800, 400)
    c.dashes = (10, 5)
    _lines(c, 800, 400)
    c.stroke()
    return s


def s055_stroke_miter_dashed(be, aa):
    s, c = _stroke_canvas(be, aa, 240, 260)
    c.dashes = (15, 5)
    _spirals(c)
    c.stroke()
    return s


def s056_stroke_star_dashed(be, aa):
    s, c = _stroke_canvas(be, aa, 300, 300)
    c.line_width = 6
    c.dashes = (12, 3)
    _stroke_star(c, 300, 300)
    c.stroke()
    return s


def s057_stroke_bezier_dashed(be, aa):
    s, c = _stroke_canvas(be, aa, 300, 300)
    c.dashes = (6, 2)
    c.move_to(19, 149)
    c.curve_to(89, 0, 209, 0, 279, 149)
    c.stroke()
    c.line_width = 6
    c.dashes = (18, 6)
    c.reset_path()
    c.move_to(19, 199)
    c.curve_to(89, 24, 209, 24, 279, 199)
    c.stroke()
    c.line_width = 10
    c.dashes = (30, 10)
    c.reset_path()
    c.move_to(19, 249)
    c.curve_to(89, 49, 209, 49, 279, 249)
    c.stroke()
    return s


def s081_stroke_hairline(be, aa):
    W = H = 300
    s = Surface.init("rgb", 600, 2100)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.hairline = True

    def done():
        c.stroke()
        c.reset_path()

    def triangle():
        m = 10
        c.move_to(m, m)
        c.line_to(W - m - 1, m)
        c.line_to(W // 2 - 1, H - m - 1)
        c.close_path()
        done()

    def square():
        m = 50
        c.move_to(m, m)
        c.line_to(W - m - 1, m)
        c.line_to(W - m - 1, H - m - 1)
        c.line_to(m, H - m - 1)
        c.close_path()
        done()

    def star():
        m, xs, ys = 20, 3, 5
        c.move_to(W // 2, m)
        c.line_to(W - m * xs - 1, H - m - 1)
        c.line_to(m, m * ys)
        c.line_to(W - m - 1, m * ys)
        c.line_to(m * xs, H - m - 1)
        c.close_path()
        done()

    def bezier():
        for y0, cy in ((149, 0), (199, 24), (249, 49)):
            c.move_to(19, y0)
            c.curve_to(89, cy, 209, cy, 279, y0)
            done()

    def arc(x, y, rx, ry):
        saved = c.get_transformation()
        c.translate(x + rx / 2, y + ry / 2)
        c.scale(rx / 2, ry / 2)
        c.arc(0, 0, 1, 0, 2 * math.pi)
        c.close_path()
        c.stroke()
        c.reset_path()
        c.set_transformation(saved)

    def circle():
        arc(W / 6, H / 6, W / 3 * 2, H / 3 * 2)

    def ellipse():
        arc(W / 3, H / 6, W / 3, H / 3 * 2)

    def dots():
        for i in range(10):
            for j in range(50):
                c.move_to(W // 6 + j * 4, W // 3 + i * 10)
                c.close_path()
            done()

    def at(tx, ty, f):
        c.translate(tx, ty)
        f()
        c.set_identity()

    triangle()
    at(300, 0, square)
    at(0, 300, star)
    at(300, 300, bezier)
    at(0, 600, circle)
    at(300, 600, ellipse)
    at(150, 900, dots)
    c.dashes = (20.0, 5.0)
    c.dash_offset = -6.0
    at(0, 1200, triangle)
    at(300, 1200, square)
    at(0, 1500, star)
    at(300, 1500, bezier)
    at(0, 1800, circle)
    at(300, 1800, ellipse)
    return s


def s032_fill_arc(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    ratio = 0.552284749831
    cy = 150
    cx, r = 100, 50
    p12 = r * ratio
    c.move_to(cx, cy - r)
    c.curve_to(cx + p12, cy - r, cx + r, cy - p12, cx + r, cy)
    c.curve_to(cx + r, cy + p12, cx + p12, cy + r, cx, cy + r)
    c.curve_to(cx - p12, cy + r, cx - r, cy + p12, cx - r, cy)
    c.curve_to(cx - r, cy - p12, cx - p12, cy - r, cx, cy - r)
    c.close_path()
    c.fill()
    cx, rM, rm = 200, 50, 25
    pM, pm = rM * ratio, rm * ratio
    c.reset_path()
    c.move_to(cx, cy - rM)
    c.curve_to(cx + pm, cy - rM, cx + rm, cy - pM, cx + rm, cy)
    c.curve_to(cx + rm, cy + pM, cx + pm, cy + rM, cx, cy + rM)
    c.curve_to(cx - pm, cy + rM, cx - rm, cy + pM, cx - rm, cy)
    c.curve_to(cx - rm, cy - pM, cx - pm, cy - rM, cx, cy - rM)
    c.close_path()
    c.fill()
    return s


def s035_arc_command(be, aa):
    s = Surface.init_pixel(_white_rgb(), 400, 400)
    c = Ctx(be, s)
    c.set_source(Pixel.rgb(0xFF, 0, 0))
    c.aa = aa
    c.line_width = 5
    c.move_to(200, 200)
    c.arc_negative(200, 200, 150, math.pi, math.pi * 1.5)
    c.close_path()
    c.fill()
    c.set_source(Pixel.rgb(0, 0, 0xFF))
    c.stroke()
    c.reset_path()
    c.move_to(175, 175)
    c.arc(175, 175, 150, math.pi, math.pi * 1.5)
    c.close_path()
    c.set_source(Pixel.rgb(0xFF, 0xFF, 0))
    c.fill()
    c.set_source(Pixel.rgb(0, 0, 0xFF))
    c.stroke()
    return s


def s042_arc_ellipses(be, aa):
    s = Surface.init("rgb", 400, 400)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 5

    def ellipse(x, y, rx, ry, reset_ctm):
        saved = c.get_transformation()
        c.reset_path()
        c.translate(x + rx / 2, y + ry / 2)
        c.scale(rx / 2, ry / 2)
        c.arc(0, 0, 1, 0, 2 * math.pi)
        if reset_ctm:
            c.set_transformation(saved)
        c.close_path()

    def user_width(lw):
        ux, uy = c.device_to_user_distance(lw, lw)
        return uy if ux < uy else ux

    c.translate(10, 10)
    ellipse(0, 0, 50, 100, True)
    c.fill()
    ellipse(100, 0, 50, 100, True)
    c.stroke()
    saved_ctm, saved_lw = c.get_transformation(), c.line_width
    ellipse(200, 0, 50, 100, False)
    c.line_width = user_width(saved_lw)
    c.stroke()
    c.set_transformation(saved_ctm)
    c.line_width = saved_lw
    saved_ctm, saved_lw = c.get_transformation(), c.line_width
    c.rotate(math.pi / 4.0)
    ellipse(300, 0, 50, 100, False)
    c.line_width = user_width(saved_lw)
    c.stroke()
    c.set_transformation(saved_ctm)
    c.line_width = saved_lw
    return s


# Zig evaluates constant expressions such as `math.pi / 6.0` at compile time
# in 128-bit precision and rounds once; the double-precision quotient
# math.pi / 6.0 is one ulp lower.
_PI = Fraction("3.14159265358979323846264338327950288419716939937510582097494459")
_PI_6 = float(_PI / 6)


def _user_width(c, lw):
    ux, uy = c.device_to_user_distance(lw, lw)
    return uy if ux < uy else ux


def s043_rect_transforms(be, aa):
    s = Surface.init("rgb", 400, 400)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 5

    def rect(x, y, h, w, reset_ctm):
        saved = c.get_transformation()
        c.reset_path()
        c.translate(x, y)
        c.scale(h, w)
        c.move_to(0, 0)
        c.line_to(1, 0)
        c.line_to(1, 1)
        c.line_to(0, 1)
        if reset_ctm:
            c.set_transformation(saved)
        c.close_path()

    c.translate(10, 10)
    rect(0, 0, 50, 100, True)
    c.fill()
    rect(100, 0, 50, 100, True)
    c.stroke()
    saved_ctm, saved_lw = c.get_transformation(), c.line_width
    rect(200, 0, 50, 100, False)
    c.line_width = _user_width(c, saved_lw)
    c.stroke()
    c.set_transformation(saved_ctm)
    c.line_width = saved_lw
    saved_ctm, saved_lw = c.get_transformation(), c.line_width
    c.rotate(math.pi / 4.0)
    rect(300, 0, 50, 100, False)
    c.line_width = _user_width(c, saved_lw)
    c.stroke()
    c.set_transformation(saved_ctm)
    c.line_width = saved_lw
    return s


def s044_line_transforms(be, aa):
    s = Surface.init("rgb", 700, 400)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 10

    def line(i, reverse, rnd):
        saved_ctm, saved_lw, saved_src = c.get_transformation(), c.line_width, c.pattern
        c.line_cap = "round" if rnd else "square"
        y = 50.0
        if reverse:
            y += 100
        if rnd:
            y += 200
        if reverse:
            c.translate(i * 100 + 25, y + 25 * math.sin(_PI_6 * i))
            c.rotate(-_PI_6 * i)
        else:
            c.translate(i * 100 + 25, y - 25 * math.sin(_PI_6 * i))
            c.rotate(_PI_6 * i)
        c.scale(2, 1)
        if reverse:
            c.move_to(0, 0)
            c.line_to(25, 0)
        else:
            c.move_to(25, 0)
            c.line_to(0, 0)
        c.line_width = _user_width(c, saved_lw)
        c.stroke()
        c.set_source(Pixel.rgb(0xF3, 0, 0))
        c.line_width = 1
        c.stroke()
        c.line_cap = "butt"
        c.pattern = saved_src
        c.line_width = saved_lw
        c.set_transformation(saved_ctm)
        c.reset_path()

    for rev, rnd in ((False, False), (True, False), (False, True), (True, True)):
        for i in range(7):
            line(float(i), rev, rnd)
    return s


def s045_round_join_transforms(be, aa):
    s = Surface.init("rgb", 800, 600)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 20
    c.line_cap = "round"
    c.line_join = "round"
    for k in range(12):
        i = float(k)
        saved_ctm, saved_lw, saved_src = c.get_transformation(), c.line_width, c.pattern
        x_off = 200 * math.fmod(i, 4.0) + 100 - 50 * math.cos(_PI_6 * i)
        y_off = 200 * math.floor(i / 4.0) + 75 - 37.5 * math.sin(_PI_6 * i)
        c.translate(x_off, y_off)
        c.rotate(_PI_6 * i)
        c.scale(2, 1)
        c.move_to(0, 0)
        c.line_to(25, 75)
        c.line_to(50, 0)
        c.line_width = _user_width(c, saved_lw)
        c.stroke()
        c.set_source(Pixel.rgb(0xF3, 0, 0))
        c.line_width = 1
        c.stroke()
        c.pattern = saved_src
        c.line_width = saved_lw
        c.set_transformation(saved_ctm)
        c.reset_path()
    return s


def s027_stroke_bezier_tolerance(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 5
    for tol, y0, cy in ((None, 149, 0), (3, 199, 24), (10, 249, 49)):
        if tol is not None:
            c.set_tolerance(tol)
        c.reset_path()
        c.move_to(19, y0)
        c.curve_to(89, cy, 209, cy, 279, y0)
        c.stroke()
    return s


def s029_stroke_lines_round_caps_tolerance(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_cap = "round"
    c.line_join = "round"
    c.line_width = 30
    for tol, y in ((None, 50), (3, 150), (10, 250)):
        if tol is not None:
            c.set_tolerance(tol)
        c.reset_path()
        c.move_to(30, y)
        c.line_to(270, y)
        c.stroke()
    return s


def s030_stroke_star_round_tolerance(be, aa):
    s = Surface.init("rgb", 900, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 30
    c.line_join = "round"
    m, sw, h, xs, ys = 20, 300, 300, 3, 5
    for tol, xo in ((None, 0.0), (3, 300.0), (10, 600.0)):
        c.reset_path()
        if tol is not None:
            c.set_tolerance(tol)
        c.move_to(xo + sw // 2, m)
        c.line_to(xo + sw - m * xs - 1, h - m - 1)
        c.line_to(xo + m, m * ys)
        c.line_to(xo + sw - m - 1, m * ys)
        c.line_to(xo + m * xs, h - m - 1)
        c.close_path()
        c.stroke()
    return s


def _poly(c, pts):
    c.move_to(*pts[0])
    for q in pts[1:]:
        c.line_to(*q)
    c.close_path()


def s033_fill_zig_mark(be, aa):
    s = Surface.init("rgba", 153, 140)
    c = Ctx(be, s)
    c.set_source(Pixel.rgb(0xF7, 0xA4, 0x1D))
    c.aa = aa
    for pts in (
        [(46, 22), (28, 44), (19, 30)],
        [(46, 22), (33, 33), (28, 44), (22, 44), (22, 95), (31, 95), (20, 100), (12, 117), (0, 117), (0, 22)],
        [(31, 95), (12, 117), (4, 106)],
        [(56, 22), (62, 36), (37, 44)],
        [(56, 22), (111, 22), (111, 44), (37, 44), (56, 32)],
        [(116, 95), (97, 117), (90, 104)],
        [(116, 95), (100, 104), (97, 117), (42, 117), (42, 95)],
        [(150, 0), (52, 117), (3, 140), (101, 22)],
        [(141, 22), (140, 40), (122, 45)],
        [(153, 22), (153, 117), (106, 117), (120, 105), (125, 95), (131, 95), (131, 45), (122, 45), (132, 36),
         (141, 22)],
        [(125, 95), (130, 110), (106, 117)],
    ):
        _poly(c, pts)
    c.fill()
    return s


def s034_stroke_cross(be, aa):
    s = Surface.init("rgb", 250, 250)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 5
    c.move_to(100, 50)
    for dx, dy in ((0, 50), (-50, 0), (0, 50), (50, 0), (0, 50), (50, 0), (0, -50), (50, 0), (0, -50), (-50, 0),
                   (0, -50)):
        c.path.rel_line_to(dx, dy)
    c.close_path()
    c.stroke()
    return s


def _polylines(c, groups):
    for pts, closed in groups:
        c.move_to(*pts[0])
        for q in pts[1:]:
            c.line_to(*q)
        if closed:
            c.close_path()


def s036_stroke_colinear(be, aa):
    s = Surface.init("rgb", 100, 240)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 4
    _polylines(c, [
        ([(40, 50), (35, 60), (30, 70), (10, 50)], False),
        ([(10, 10), (20, 20), (30, 30), (40, 10)], False),
        ([(90, 50), (85, 60), (80, 70), (60, 50)], True),
        ([(60, 10), (70, 20), (80, 30), (90, 10)], True),
        ([(10, 90), (25, 100), (40, 110)], False),
        ([(10, 150), (25, 140), (40, 130)], False),
        ([(90, 90), (75, 100), (60, 110)], False),
        ([(90, 150), (75, 140), (60, 130)], False),
        ([(10, 170), (30, 190), (20, 180), (40, 170)], False),
        ([(90, 170), (70, 190), (80, 180), (60, 170)], False),
        ([(40, 210), (30, 230), (20, 220), (10, 210)], False),
        ([(60, 210), (70, 230), (80, 220), (90, 210)], False),
    ])
    c.stroke()
    return s


def s037_stroke_join_overlap(be, aa):
    s = Surface.init("rgb", 200, 200)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 5
    c.miter_limit = 4
    _polylines(c, [
        ([(10, 10), (50, 90), (35, 50)], False),
        ([(190, 10), (150, 90), (165, 50)], False),
        ([(10, 190), (50, 110), (35, 150)], False),
        ([(190, 190), (150, 110), (165, 150)], False),
    ])
    c.stroke()
    return s


def s038_stroke_zero_length(be, aa):
    s = Surface.init("rgb", 60, 60)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 10
    c.line_cap = "round"
    c.move_to(10, 10)
    c.close_path()
    c.move_to(30, 30)
    c.line_to(30, 30)
    c.line_to(30, 30)
    c.close_path()
    c.move_to(50, 50)
    c.stroke()
    return s


def s039_stroke_paint_extent_dontclip(be, aa):
    s = Surface.init("rgb", 50, 80)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 5
    _polylines(c, [([(40, 50), (35, 60), (30, 70), (10, 50)], False)])
    c.stroke()
    return s


def s040_stroke_corner_symmetrical(be, aa):
    s = Surface.init("rgb", 18, 36)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.move_to(0, 0)
    c.line_to(18, 36)
    c.stroke()
    return s


def s041_stroke_noop_lineto(be, aa):
    s = Surface.init("rgb", 18, 36)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    _polylines(c, [([(9, 0), (9, 9), (0, 18), (0, 18)], False)])
    c.stroke()
    return s


def s073_stroke_sameclose(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    m = 50
    _polylines(c, [([(m, m), (300 - m - 1, m), (300 - m - 1, 300 - m - 1), (m, 300 - m - 1), (m, m)], True)])
    c.stroke()
    return s


def s078_double_close(be, aa):
    s = Surface.init_pixel(Pixel.from_color(Color.rgb(0.33, 0.33, 0.33)), 300, 300)
    c = Ctx(be, s)
    c.aa = aa
    c.move_to(49, 49)
    c.line_to(250, 49)
    c.line_to(250, 250)
    c.line_to(49, 250)
    c.close_path()
    c.close_path()
    c.set_source(Pixel.rgb(0, 0xFF, 0))
    c.fill()
    c.set_source(Pixel.rgb(0xFF, 0, 0xFF))
    c.stroke()
    return s


def s058_stroke_misc_dashes(be, aa):
    s = Surface.init("rgb", 600, 2000)
    c = Ctx(be, s)
    c.set_source(_white_rgb())
    c.aa = aa
    c.line_width = 3
    c.dashes = (25.0, 5.0)

    def at(tx, ty):
        c.set_identity()
        c.translate(tx, ty)

    def line(pts, close=False):
        c.move_to(*pts[0])
        for q in pts[1:]:
            c.line_to(*q)
        if close:
            c.close_path()
        c.stroke()
        c.reset_path()

    c.translate(50, 50)
    line([(100, 0), (200, 200), (0, 200)], True)
    at(350, 50)
    line([(0, 0), (0, 200), (200, 200), (200, 0)], True)
    d = 200
    at(50 + d / 2, 350 + d / 2)  # circle
    c.scale(d / 2, d / 2)
    c.arc(0, 0, 1, 0, 2 * math.pi)
    c.set_identity()
    c.stroke()
    c.reset_path()
    at(350 + d / 2, 350 + d / 2)  # fill + stroke
    c.scale(d / 2, d / 2)
    c.arc(0, 0, 1, 0, 2 * math.pi)
    c.close_path()
    c.set_identity()
    c.set_source(Pixel.rgb(0xAA, 0xAA, 0xAA))
    c.fill()
    c.set_source(_white_rgb())
    c.stroke()
    c.reset_path()
    elw = 6.0  # ellipse, no transform on the stroke
    c.line_width = elw
    xd, yd = 100, 200
    at(100 + xd / 2, 650 + yd / 2)
    c.scale(xd / 2, yd / 2)
    c.arc(0, 0, 1, 0, 2 * math.pi)
    c.set_identity()
    c.stroke()
    c.reset_path()
    at(400 + xd / 2, 650 + yd / 2)  # ellipse, transform on the stroke
    c.scale(xd / 2, yd / 2)
    c.arc(0, 0, 1, 0, 2 * math.pi)
    c.line_width = _user_width(c, elw)
    c.stroke()
    c.set_identity()
    c.reset_path()
    at(50, 950)  # square through the transform
    c.scale(200, 200)
    c.move_to(0, 0)
    c.line_to(0, 1)
    c.line_to(1, 1)
    c.line_to(1, 0)
    c.close_path()
    c.line_width = _user_width(c, elw)
    c.stroke()
    c.set_identity()
    c.reset_path()
    c.line_width = 3  # odd dash arrays
    at(350, 950)
    c.dashes = (28.0,)
    line([(0, 0), (200, 0)])
    at(350, 990)
    c.dashes = (25.0, 5.0, 3.0)
    line([(0, 0), (200, 0)])
    c.line_width = 10  # capping
    for cap, y in (("round", 1030), ("square", 1070), ("butt", 1110)):
        c.line_cap = cap
        at(350, y)
        c.dashes = (28.0,)
        line([(0, 0), (200, 0)])
    c.line_cap = "round"  # dots
    at(350, 1150)
    c.dashes = (0.0, 20.0)
    line([(0, 0), (200, 0)])
    c.line_cap = "square"  # squares aligned to the slope
    at(50, 1250)
    c.dashes = (0.0, 20.0)
    c.move_to(0, 0)
    c.line_to(0, 200)
    c.move_to(20, 0)
    c.line_to(200, 200)
    c.stroke()
    c.reset_path()
    c.line_cap = "butt"  # offsets
    c.line_width = 3
    c.set_identity()
    c.dashes = (25.0,)
    c.dash_offset = 12.5
    c.translate(350, 1225)
    line([(0, 0), (200, 0), (200, 100), (0, 100)], True)
    at(350, 1350)
    c.dash_offset = -12.5
    line([(0, 0), (200, 0), (200, 100), (0, 100)], True)
    c.line_width = 10
    c.set_identity()
    c.dashes = ()
    c.dash_offset = 0.0
    c.translate(150, 1550)
    line([(0, 0), (300, 0)])
    at(150, 1570)
    c.dashes = (30.0, 10.0)
    c.dash_offset = 0.0
    line([(0, 0), (300, 0)])
    for y, off in ((1590, 30.0), (1610, -30.0), (1630, 10.0)):
        at(150, y)
        c.dash_offset = off
        line([(0, 0), (300, 0)])
    c.set_source(Pixel.rgba(127, 0, 0, 127))  # RGBA{255, 0, 0, 127}.multiply()
    at(150, 1590)
    c.dashes = ()
    c.dash_offset = 0.0
    for y, dx in ((1590, -30), (1610, 30), (1630, -10)):
        at(150, y)
        c.move_to(0, 0)
        c.path.rel_line_to(dx, 0)
        c.stroke()
        c.reset_path()
    c.set_source(_white_rgb())  # octagon
    at(200, 1725)
    c.dash_offset = 0.0
    c.dashes = (180.0, 30.0)
    line([(136.737609507049, 188.692435121084), (63.2623904929514, 188.692435121084),
          (11.3075648789165, 136.737609507049), (11.3075648789165, 63.2623904929514),
          (63.2623904929513, 11.3075648789165), (136.737609507049, 11.3075648789165),
          (188.692435121084, 63.2623904929513), (188.692435121084, 136.737609507049)], True)
    return s


def _oob_scene(draws):
    def scene(be, aa):
        s = Surface.init_pixel(Pixel.from_color(Color.rgb(0.33, 0.33, 0.33)), 300, 300)
        c = Ctx(be, s)
        c.aa = aa
        for k, (tx, ty, pts, first_line) in enumerate(draws):
            c.reset_path()
            c.set_identity()
            c.translate(tx, ty)
            (c.line_to if first_line else c.move_to)(*pts[0])
            for q in pts[1:]:
                c.line_to(*q)
            c.close_path()
            c.set_source(Pixel.rgb(0, 0xFF, 0))
            c.fill()
            c.set_source(Pixel.rgb(0xFF, 0, 0xFF))
            c.stroke()
        return s
    return scene


_W, _CX, _M = 300, 150, 10
s075_oob_draw_corners = _oob_scene([
    (-_M, -_M, [(_CX, _CX), (-_CX, _CX), (_CX, -_CX)], True),
    (_M, -_M, [(_CX, _CX), (_W + _CX, _CX), (_W + _CX, -_CX), (_CX, -_CX)], False),
    (-_M, _M, [(_CX, _CX), (-_CX, _CX), (-_CX, _W + _CX), (_CX, _W + _CX)], False),
    (_M, _M, [(_CX, _CX), (_W + _CX, _CX), (_W + _CX, _W + _CX), (_CX, _W + _CX)], False),
])
s076_oob_draw_sides = _oob_scene([
    (0, -_M, [(_CX - _M, _CX), (_CX - _M, -_CX), (_CX + _M, -_CX), (_CX + _M, _CX)], False),
    (0, _M, [(_CX - _M, _CX), (_CX - _M, _W + _CX), (_CX + _M, _W + _CX), (_CX + _M, _CX)], False),
    (-_M, 0, [(_CX, _CX - _M), (-_CX, _CX - _M), (-_CX, _CX + _M), (_CX, _CX + _M)], False),
    (_M, 0, [(_CX, _CX - _M), (_W + _CX, _CX - _M), (_W + _CX, _CX + _M), (_CX, _CX + _M)], False),
])


def s077_oob_draw_full_outside(be, aa):
    s = Surface.init("rgb", 300, 300)
    c = Ctx(be, s)
    c.aa = aa
    for cx, cy in ((-300, -300), (600, -300), (600, 600), (-300, 600), (-300, 150), (600, 150), (150, -300),
                   (150, 600)):
        c.reset_path()
        c.set_identity()
        c.translate(cx, cy)
        c.move_to(cx - 20, cy - 20)
        c.line_to(cx + 20, cy - 20)
        c.line_to(cx + 20, cy + 20)
        c.line_to(cx - 20, cy + 20)
        c.close_path()
        c.set_source(Pixel.rgb(0, 0xFF, 0))
        c.fill()
        c.set_source(Pixel.rgb(0xFF, 0, 0xFF))
        c.stroke()
    return s


_HAIRLINE_CLIP_CASES = [  # (x0, y0, x1, y1) on a 100x100 canvas
    (-25, 50, 75, 60), (25, 50, 125, 60), (-25, 50, 75, 50), (25, 50, 125, 50),
    (25, -50, 75, 50), (25, 50, 75, 150), (-25, -50, -75, -150), (125, 150, 175, 250),
    (50, -25, 60, 75), (50, 25, 60, 125), (50, -25, 50, 75), (50, 25, 50, 125),
    (-50, 25, 50, 75), (50, 25, 150, 75), (-50, -25, -150, -75), (150, 125, 250, 175),
]


def s082_stroke_hairline_clip(be, aa):
    from z2d_gb300.types import StrokeOptions
    s = Surface.init("rgb", 200, len(_HAIRLINE_CLIP_CASES) // 2 * 100)
    for idx, (x0, y0, x1, y1) in enumerate(_HAIRLINE_CLIP_CASES):
        on = 0x20 * (((idx // 2) & 1) ^ (idx % 2))
        src = Surface.init_pixel(Pixel.rgb(on, on, on), 100, 100)
        p = Path()
        p.move_to(x0, y0)
        p.line_to(x1, y1)
        rc = be.stroke(src, Pattern.from_pixel(_white_rgb()), p.nodes, StrokeOptions(anti_aliasing=aa, hairline=True))
        assert rc == abi.OK
        rc = be.composite(s, idx % 2 * 100, idx // 2 * 100, [Operation("src", src=src)])
        assert rc == abi.OK
    return s


STROKE_SCENES = {
    "008_stroke_triangle": s008_stroke_triangle,
    "009_stroke_square": s009_stroke_square,
    "010_stroke_trapezoid": s010_stroke_trapezoid,
    "011_stroke_star": s011_stroke_star,
    "012_stroke_bezier": s012_stroke_bezier,
    "014_stroke_lines": s014_stroke_lines,
    "015_stroke_miter": s015_stroke_miter,
    "017_stroke_star_round": s017_stroke_star_round,
    "018_stroke_square_spiral_round": s018_stroke_square_spiral_round,
    "019_stroke_bevel_miterlimit": s019_stroke_bevel_miterlimit,
    "020_stroke_lines_round_caps": s020_stroke_lines_round_caps,
    "021_stroke_lines_square_caps": s021_stroke_lines_square_caps,
    "022_stroke_lines_butt_caps": s022_stroke_lines_butt_caps,
    "054_stroke_lines_dashed": s054_stroke_lines_dashed,
    "055_stroke_miter_dashed": s055_stroke_miter_dashed,
    "056_stroke_star_dashed": s056_stroke_star_dashed,
    "057_stroke_bezier_dashed": s057_stroke_bezier_dashed,
    "027_bezier_tolerance": s027_stroke_bezier_tolerance,
    "029_stroke_lines_round_caps_tolerance": s029_stroke_lines_round_caps_tolerance,
    "030_stroke_star_round_tolerance": s030_stroke_star_round_tolerance,
    "034_stroke_cross": s034_stroke_cross,
    "035_arc_command": s035_arc_command,
    "036_stroke_colinear": s036_stroke_colinear,
    "037_stroke_join_overlap": s037_stroke_join_overlap,
    "038_stroke_zero_length": s038_stroke_zero_length,
    "039_stroke_paint_extent_dontclip": s039_stroke_paint_extent_dontclip,
    "040_stroke_corner_symmetrical": s040_stroke_corner_symmetrical,
    "041_stroke_noop_lineto": s041_stroke_noop_lineto,
    "058_stroke_misc_dashes": s058_stroke_misc_dashes,
    "059_stroke_star_gradient": s059_stroke_star_gradient,
    "073_stroke_sameclose": s073_stroke_sameclose,
    "075_oob_draw_corners": s075_oob_draw_corners,
    "076_oob_draw_sides": s076_oob_draw_sides,
    "077_oob_draw_full_outside": s077_oob_draw_full_outside,
    "078_double_close": s078_double_close,
    "042_arc_ellipses": s042_arc_ellipses,
    "043_rect_transforms": s043_rect_transforms,
    "044_line_transforms": s044_line_transforms,
    "045_round_join_transforms": s045_round_join_transforms,
    "081_stroke_hairline": s081_stroke_hairline,
    "082_stroke_hairline_clip": s082_stroke_hairline_clip,
}

FILL_SCENES = {
    "003_fill_triangle": s003_fill_triangle,
    "004_fill_square": s004_fill_square,
    "005_fill_trapezoid": s005_fill_trapezoid,
    "006_fill_star_even_odd": s006_fill_star_even_odd,
    "007_fill_bezier": s007_fill_bezier,
    "013_fill_combined": s013_fill_combined,
    "016_fill_star_non_zero": s016_fill_star_non_zero,
    "024_fill_triangle_direct_cross_format": s024_fill_triangle_direct_cross_format,
    "025_fill_diamond_clipped": s025_fill_diamond_clipped,
    "026_fill_triangle_full": s026_fill_triangle_full,
    "028_fill_bezier_tolerance": s028_fill_bezier_tolerance,
    "031_fill_quad_bezier": s031_fill_quad_bezier,
    "046_fill_triangle_alpha": s046_fill_triangle_alpha,
    "047_fill_triangle_alpha_gray": _alpha_tri("alpha8", Pixel.alpha8(119)),
    "048_fill_triangle_static": s048_fill_triangle_static,
    "049_fill_triangle_alpha4_gray": _alpha_tri("alpha4", Pixel.alpha4(7)),
    "050_fill_triangle_alpha2_gray": _alpha_tri("alpha2", Pixel.alpha2(2)),
    "051_fill_triangle_alpha1_gray": _alpha_tri("alpha1", Pixel.alpha1(1)),
    "052_fill_triangle_alpha4_gray_scaledown": _alpha_tri("alpha4", Pixel.alpha8(119)),
    "053_fill_triangle_alpha8_gray_scaleup": _alpha_tri("alpha8", Pixel.alpha4(7)),
    "079_fill_degenerate_lineto": s079_fill_degenerate_lineto,
    "032_fill_arc": s032_fill_arc,
    "033_fill_zig_mark": s033_fill_zig_mark,
    "064_radial_source": s064_radial_source,
    "066_conic_pie_gradient": s066_conic_pie_gradient,
    "067_gradient_transforms": s067_gradient_transforms,
    "069_gradient_dither_context": s069_gradient_dither_context,
    "070_compositor_ops": s070_compositor_ops,
}

COMPOSITOR_SCENES = {
    "061_linear_gradient": s061_linear_gradient,
    "062_hsl_gradient": s062_hsl_gradient,
    "063_radial_gradient": s063_radial_gradient,
    "065_conic_gradient": s065_conic_gradient,
    "068_gradient_deband": s068_gradient_deband,
}

# AA mode -> golden suffix (spec/main_spec.zig:564-634, 772-831)
AA_SUFFIX = {"none": "_pixelated", "supersample_4x": "_smooth", "multisample_4x": "_smooth_multisample"}
