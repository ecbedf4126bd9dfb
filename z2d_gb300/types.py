"""Host-side mirror of z2d's pixel, color, gradient, pattern and option types.

These are plain descriptions that marshal into the C ABI structs of
include/z2dgpu.h.  Each class cites the z2d type it mirrors.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

import numpy as np

from . import abi


def _fmt(f: Union[int, str]) -> int:
    return abi.FORMAT_NAMES.index(f) if isinstance(f, str) else int(f)


def _op(o: Union[int, str]) -> int:
    return abi.OP[o] if isinstance(o, str) else int(o)


# --------------------------------------------------------------------------
# Pixels                                            src/pixel.zig:101-142
# --------------------------------------------------------------------------
@dataclass(frozen=True)
class Pixel:
    """A pixel in its own format (pixel.Pixel).  For alpha4/2/1, `a` is the
    raw 4/2/1-bit value."""
    format: int
    r: int = 0
    g: int = 0
    b: int = 0
    a: int = 0

    @staticmethod
    def rgb(r, g, b):
        return Pixel(abi.FORMAT_RGB, r, g, b, 0)

    @staticmethod
    def xrgb(r, g, b):
        return Pixel(abi.FORMAT_XRGB, r, g, b, 0)

    @staticmethod
    def rgba(r, g, b, a):
        return Pixel(abi.FORMAT_RGBA, r, g, b, a)

    @staticmethod
    def argb(r, g, b, a):
        return Pixel(abi.FORMAT_ARGB, r, g, b, a)

    @staticmethod
    def alpha8(a):
        return Pixel(abi.FORMAT_ALPHA8, 0, 0, 0, a)

    @staticmethod
    def alpha4(a):
        return Pixel(abi.FORMAT_ALPHA4, 0, 0, 0, a)

    @staticmethod
    def alpha2(a):
        return Pixel(abi.FORMAT_ALPHA2, 0, 0, 0, a)

    @staticmethod
    def alpha1(a):
        return Pixel(abi.FORMAT_ALPHA1, 0, 0, 0, a)

    @staticmethod
    def from_color(color: "Color") -> "Pixel":
        """Pixel.fromColor (src/pixel.zig:119-121) for linear and sRGB colors:
        sRGB gamma removed (pow 2.2, rounded to f32), round(255 x), then
        integer premultiply (src/color.zig:272-289)."""
        if color.space == abi.COLOR_SRGB:  # SRGB.removeGamma: pow(x, 2.2) in f32
            lin = [float(np.float32(math.pow(float(c), float(np.float32(2.2))))) if c not in (0.0, 1.0) else c
                   for c in color.c[:3]] + [color.c[3]]
        elif color.space == abi.COLOR_LINEAR_RGB:
            lin = list(color.c)
        else:
            raise NotImplementedError("from_color: HSL colors are not converted host-side")
        v = [int(math.floor(float(np.float32(255.0) * np.float32(c)) + 0.5)) for c in lin]
        r, g, b, a = v
        return Pixel.rgba(r * a // 255, g * a // 255, b * a // 255, a)

    def to_abi(self) -> abi.z2d_pixel:
        return abi.z2d_pixel(self.format, self.r, self.g, self.b, self.a)

    def can_demultiply(self) -> bool:
        """RGBA_T.canDemultiply (src/pixel.zig:504-514)."""
        if self.format not in (abi.FORMAT_ARGB, abi.FORMAT_RGBA) or self.a == 0:
            return True
        return all(c * 255 // self.a <= 255 for c in (self.r, self.g, self.b))


# --------------------------------------------------------------------------
# Colors                                              src/color.zig:41-93
# --------------------------------------------------------------------------
def _clamp01(v: float) -> float:
    v = float(np.float32(v))
    return min(max(v, 0.0), 1.0)


@dataclass(frozen=True)
class Color:
    """color.Color as stored after Color.init (clamped, hue wrapped)."""
    space: int
    c: tuple

    @staticmethod
    def rgb(r, g, b, a=1.0):
        return Color(abi.COLOR_LINEAR_RGB, tuple(_clamp01(x) for x in (r, g, b, a)))

    @staticmethod
    def srgb(r, g, b, a=1.0):
        return Color(abi.COLOR_SRGB, tuple(_clamp01(x) for x in (r, g, b, a)))

    @staticmethod
    def hsl(h, s, l, a=1.0):
        """HSL.init (src/color.zig:412-419): hue wrapped by @mod when
        outside [0, 360]."""
        h = float(np.float32(h))
        if h < 0 or h > 360:
            r = math.fmod(h, 360.0)
            h = math.fmod(r + 360.0, 360.0) if h < 0 else r
            h = float(np.float32(h))
        return Color(abi.COLOR_HSL, (h, _clamp01(s), _clamp01(l), _clamp01(a)))

    def to_abi(self) -> abi.z2d_color:
        col = abi.z2d_color()
        col.space = self.space
        for i in range(4):
            col.c[i] = self.c[i]
        return col


# --------------------------------------------------------------------------
# Transformation                                     src/Transformation.zig
# --------------------------------------------------------------------------
IDENTITY = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)  # ax, by, cx, dy, tx, ty


def transformation_inverse(m: Sequence[float]) -> tuple:
    """Transformation.inverse (src/Transformation.zig:103-161)."""
    ax, by, cx, dy, tx, ty = (float(v) for v in m)
    if by == 0 and cx == 0:
        if ax == 0 or dy == 0:
            raise ValueError("InvalidMatrix")
        if ax != 1 or dy != 1:
            return (1 / ax, 0.0, 0.0, 1 / dy, -tx / ax, -ty / dy)
        return (1.0, 0.0, 0.0, 1.0, -tx, -ty)
    det = ax * dy - by * cx
    if det == 0:
        raise ValueError("InvalidMatrix")
    adj = (dy, -by, -cx, ax, by * ty - dy * tx, cx * tx - ax * ty)
    s = 1 / det
    return tuple(v * s for v in adj)


# --------------------------------------------------------------------------
# Gradients                                         src/gradient.zig:42-265
# --------------------------------------------------------------------------
class Gradient:
    """gradient.Gradient: linear, radial or conic, with stops."""

    def __init__(self, type: str, geom: Sequence[float], method: Union[str, int] = "linear_rgb",
                 polar: str = "shorter"):
        self.type = {"linear": abi.GRADIENT_LINEAR, "radial": abi.GRADIENT_RADIAL,
                     "conic": abi.GRADIENT_CONIC}[type]
        g = [float(v) for v in geom] + [0.0] * (6 - len(geom))
        self.geom = tuple(g[:6])
        if isinstance(method, int):
            self.method = method
        elif method == "linear_rgb":
            self.method = abi.INTERP_LINEAR_RGB
        elif method == "srgb":
            self.method = abi.INTERP_SRGB
        elif method == "hsl":
            self.method = abi.INTERP_HSL[polar]
        else:
            raise ValueError(method)
        self.stops: List[tuple] = []
        self.transform = IDENTITY

    @staticmethod
    def linear(x0, y0, x1, y1, **kw):
        return Gradient("linear", (x0, y0, x1, y1), **kw)

    @staticmethod
    def radial(inner_x, inner_y, inner_r, outer_x, outer_y, outer_r, **kw):
        return Gradient("radial", (inner_x, inner_y, inner_r, outer_x, outer_y, outer_r), **kw)

    @staticmethod
    def conic(x, y, angle, **kw):
        return Gradient("conic", (x, y, angle), **kw)

    def add_stop(self, offset: float, color: Color) -> "Gradient":
        """Gradient.addStop; clamping and ordering happen in the library
        exactly as Stop.List.addAssumeCapacity does (src/gradient.zig:797-811)."""
        self.stops.append((float(np.float32(offset)), color))
        return self

    def set_transformation(self, m: Sequence[float]) -> None:
        """setTransformation stores the inverse (src/gradient.zig:322-324)."""
        self.transform = transformation_inverse(m)

    def to_abi(self, keep: list) -> abi.z2d_gradient:
        arr = (abi.z2d_stop * max(1, len(self.stops)))()
        for i, (off, col) in enumerate(self.stops):
            arr[i].offset = off
            arr[i].color = col.to_abi()
        g = abi.z2d_gradient()
        g.type, g.method, g.n_stops = self.type, self.method, len(self.stops)
        for i in range(6):
            g.geom[i] = self.geom[i]
            g.transform[i] = self.transform[i]
        g.stops = C.cast(arr, C.POINTER(abi.z2d_stop))
        keep.extend([arr, g])
        return g


# --------------------------------------------------------------------------
# Patterns and dither                  src/pattern.zig:32-50, src/Dither.zig
# --------------------------------------------------------------------------
@dataclass
class Pattern:
    kind: int
    pixel: Optional[Pixel] = None
    gradient: Optional[Gradient] = None
    dither_type: int = abi.DITHER_NONE
    dither_source: int = abi.DITHER_SRC_PIXEL
    dither_scale: int = 8
    dither_color: Optional[Color] = None

    @staticmethod
    def from_pixel(px: Pixel) -> "Pattern":
        return Pattern(abi.PATTERN_PIXEL, pixel=px)

    @staticmethod
    def from_gradient(g: Gradient) -> "Pattern":
        return Pattern(abi.PATTERN_GRADIENT, gradient=g)

    @staticmethod
    def dither(type: str, source: Union[Pixel, Gradient, Color], scale: int = 8) -> "Pattern":
        t = {"none": abi.DITHER_NONE, "bayer": abi.DITHER_BAYER, "blue_noise": abi.DITHER_BLUE_NOISE}[type]
        if isinstance(source, Pixel):
            return Pattern(abi.PATTERN_DITHER, pixel=source, dither_type=t,
                           dither_source=abi.DITHER_SRC_PIXEL, dither_scale=scale)
        if isinstance(source, Gradient):
            return Pattern(abi.PATTERN_DITHER, gradient=source, dither_type=t,
                           dither_source=abi.DITHER_SRC_GRADIENT, dither_scale=scale)
        return Pattern(abi.PATTERN_DITHER, dither_color=source, dither_type=t,
                       dither_source=abi.DITHER_SRC_COLOR, dither_scale=scale)

    def to_abi(self, keep: list) -> abi.z2d_pattern:
        p = abi.z2d_pattern()
        p.kind = self.kind
        if self.pixel is not None:
            p.pixel = self.pixel.to_abi()
        if self.gradient is not None:
            p.gradient = C.pointer(self.gradient.to_abi(keep))
        p.dither_type = self.dither_type
        p.dither_source = self.dither_source
        p.dither_scale = self.dither_scale
        if self.dither_color is not None:
            p.dither_color = self.dither_color.to_abi()
        keep.append(p)
        return p


def wrap_dither(pattern: Pattern, dither: str, surface_format: int) -> Pattern:
    """Context.wrapDither (src/Context.zig:679-699)."""
    if dither == "none" or pattern.kind == abi.PATTERN_DITHER:
        return pattern
    scale = {abi.FORMAT_ALPHA1: 1, abi.FORMAT_ALPHA2: 2, abi.FORMAT_ALPHA4: 4}.get(surface_format, 8)
    src = pattern.pixel if pattern.kind == abi.PATTERN_PIXEL else pattern.gradient
    return Pattern.dither(dither, src, scale)


# --------------------------------------------------------------------------
# Options                                 src/painter.zig:28-48, options.zig
# --------------------------------------------------------------------------
@dataclass
class FillOptions:
    anti_aliasing: str = "default"
    fill_rule: str = "non_zero"
    operator: Union[str, int] = "src_over"
    precision: str = "integer"
    tolerance: float = 0.1

    def to_abi(self) -> abi.z2d_fill_opts:
        o = abi.z2d_fill_opts()
        o.anti_aliasing = {"none": abi.AA_NONE, "default": abi.AA_DEFAULT,
                           "multisample_4x": abi.AA_MULTISAMPLE_4X,
                           "supersample_4x": abi.AA_SUPERSAMPLE_4X}[self.anti_aliasing]
        o.fill_rule = {"non_zero": abi.FILL_NON_ZERO, "even_odd": abi.FILL_EVEN_ODD}[self.fill_rule]
        o.op = _op(self.operator)
        o.precision = {"integer": abi.PRECISION_INTEGER, "float": abi.PRECISION_FLOAT}[self.precision]
        o.tolerance = float(self.tolerance)
        return o


@dataclass
class StrokeOptions:
    """painter.StrokeOptions (src/painter.zig:145-195)."""
    anti_aliasing: str = "default"
    dashes: Sequence[float] = ()
    dash_offset: float = 0.0
    line_cap: str = "butt"
    line_join: str = "miter"
    line_width: float = 2.0
    miter_limit: float = 10.0
    operator: Union[str, int] = "src_over"
    precision: str = "integer"
    tolerance: float = 0.1
    transformation: Sequence[float] = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)  # ax, by, cx, dy, tx, ty
    hairline: bool = False

    def to_abi(self, keep: list) -> abi.z2d_stroke_opts:
        o = abi.z2d_stroke_opts()
        o.anti_aliasing = {"none": abi.AA_NONE, "default": abi.AA_DEFAULT,
                           "multisample_4x": abi.AA_MULTISAMPLE_4X,
                           "supersample_4x": abi.AA_SUPERSAMPLE_4X}[self.anti_aliasing]
        o.line_join = {"miter": abi.JOIN_MITER, "round": abi.JOIN_ROUND, "bevel": abi.JOIN_BEVEL}[self.line_join]
        o.line_cap = {"butt": abi.CAP_BUTT, "round": abi.CAP_ROUND, "square": abi.CAP_SQUARE}[self.line_cap]
        o.op = _op(self.operator)
        o.precision = {"integer": abi.PRECISION_INTEGER, "float": abi.PRECISION_FLOAT}[self.precision]
        o.hairline = 1 if self.hairline else 0
        o.line_width = float(self.line_width)
        o.miter_limit = float(self.miter_limit)
        o.tolerance = float(self.tolerance)
        o.dash_offset = float(self.dash_offset)
        for i, v in enumerate(self.transformation):
            o.transformation[i] = float(v)
        if len(self.dashes):
            arr = (C.c_double * len(self.dashes))(*map(float, self.dashes))
            keep.append(arr)
            o.dashes = C.cast(arr, C.POINTER(C.c_double))
            o.n_dashes = len(self.dashes)
        return o


# --------------------------------------------------------------------------
# Compositor operations          SurfaceCompositor.Operation (compositor.zig:223-284)
# --------------------------------------------------------------------------
@dataclass
class Param:
    """Operation.Param: none, pixel, gradient, dither (a Pattern), or surface."""
    pattern: Optional[Pattern] = None
    surface: Optional[object] = None

    @property
    def kind(self) -> int:
        if self.surface is not None:
            return abi.PARAM_SURFACE
        if self.pattern is None:
            return abi.PARAM_NONE
        return {abi.PATTERN_PIXEL: abi.PARAM_PIXEL, abi.PATTERN_GRADIENT: abi.PARAM_GRADIENT,
                abi.PATTERN_DITHER: abi.PARAM_DITHER}[self.pattern.kind]


def as_param(x) -> Param:
    if x is None:
        return Param()
    if isinstance(x, Param):
        return x
    if isinstance(x, Pattern):
        return Param(pattern=x)
    if isinstance(x, Pixel):
        return Param(pattern=Pattern.from_pixel(x))
    if isinstance(x, Gradient):
        return Param(pattern=Pattern.from_gradient(x))
    return Param(surface=x)


@dataclass
class Operation:
    operator: Union[str, int]
    dst: object = None
    src: object = None

    def to_abi(self, keep: list, surface_to_abi) -> abi.z2d_operation:
        o = abi.z2d_operation()
        o.op = _op(self.operator)
        for name in ("dst", "src"):
            prm = as_param(getattr(self, name))
            out = getattr(o, name)
            out.kind = prm.kind
            if prm.surface is not None:
                s = surface_to_abi(prm.surface)
                keep.append(s)
                out.surface = C.pointer(s)
            elif prm.pattern is not None:
                out.pattern = prm.pattern.to_abi(keep)
        return o


def nodes_to_abi(nodes) -> "C.Array":
    """Accepts a sequence of (tag, p0..p5) tuples, a structured/2-D numpy
    array, or a ctypes array of z2d_node."""
    if isinstance(nodes, C.Array):
        return nodes
    if isinstance(nodes, np.ndarray):
        if nodes.dtype == NODE_DTYPE:
            arr = (abi.z2d_node * max(1, len(nodes)))()
            C.memmove(arr, nodes.ctypes.data, nodes.nbytes)
            return arr
        raise TypeError("node arrays must use NODE_DTYPE")
    arr = (abi.z2d_node * max(1, len(nodes)))()
    for i, nd in enumerate(nodes):
        arr[i].tag = nd[0]
        for j, v in enumerate(nd[1:7]):
            arr[i].p[j] = v
    return arr


# numpy view of z2d_node (56 bytes)
NODE_DTYPE = np.dtype([("tag", "<i4"), ("_pad", "<i4"), ("p", "<f8", (6,))])
assert NODE_DTYPE.itemsize == C.sizeof(abi.z2d_node) == 56
