"""Path builder producing the node arrays painter.fill consumes.

Mirrors z2d's Path (src/Path.zig:116-262, 447-477): coordinates are clamped
to the i24 range (clampI24, :570), transformed by the current matrix at
insertion, a repeated move_to to the same point is dropped, and close()
appends close_path plus a move_to back to the subpath's initial point.
"""
from __future__ import annotations

import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import abi
from .types import IDENTITY, NODE_DTYPE

_I24_MIN, _I24_MAX = -(1 << 23), (1 << 23) - 1


def _clamp_i24(v: float) -> float:
    return min(max(float(v), _I24_MIN), _I24_MAX)


# ---------------------------------------------------------------- Transformation
# src/Transformation.zig: (ax, by, cx, dy, tx, ty) tuples.
def tf_mul(a: Sequence[float], b: Sequence[float]) -> tuple:
    """Transformation.mul (Transformation.zig:68-89): a · b."""
    aax, aby, acx, ady, atx, aty = a
    bax, bby, bcx, bdy, btx, bty = b
    return (aax * bax + aby * bcx, aax * bby + aby * bdy, acx * bax + ady * bcx, acx * bby + ady * bdy,
            aax * btx + aby * bty + atx, acx * btx + ady * bty + aty)


def tf_translate(a, tx: float, ty: float) -> tuple:
    return tf_mul(a, (1.0, 0.0, 0.0, 1.0, float(tx), float(ty)))


def tf_scale(a, sx: float, sy: float) -> tuple:
    return tf_mul(a, (float(sx), 0.0, 0.0, float(sy), 0.0, 0.0))


def tf_rotate(a, angle: float) -> tuple:
    s, c = math.sin(angle), math.cos(angle)
    return tf_mul(a, (c, -s, s, c, 0.0, 0.0))


def tf_inverse(a) -> tuple:
    """Transformation.inverse (Transformation.zig:103-162); raises on a
    matrix that cannot be inverted."""
    ax, by, cx, dy, tx, ty = a
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
    sc = 1 / det
    return tuple(v * sc for v in adj)


def tf_distance(a, x: float, y: float) -> tuple:
    """Transformation.userToDeviceDistance: (x, y) through a without translation."""
    return (a[0] * x + a[1] * y, a[2] * x + a[3] * y)


# ---------------------------------------------------------------------- arcs
# src/internal/arc.zig (after cairo-arc.c): circular arcs as cubic splines.
_MAX_FULL_CIRCLES = 65536
_ARC_TABLE = [  # (angle, error) of arc_max_angle_for_tolerance_normalized (arc.zig:43-56)
    (math.pi / 1.0, 0.0185185185185185036127), (math.pi / 2.0, 0.000272567143730179811158),
    (math.pi / 3.0, 2.38647043651461047433e-05), (math.pi / 4.0, 4.2455377443222443279e-06),
    (math.pi / 5.0, 1.11281001494389081528e-06), (math.pi / 6.0, 3.72662000942734705475e-07),
    (math.pi / 7.0, 1.47783685574284411325e-07), (math.pi / 8.0, 6.63240432022601149057e-08),
    (math.pi / 9.0, 3.2715520137536980553e-08), (math.pi / 10.0, 1.73863223499021216974e-08),
    (math.pi / 11.0, 9.81410988043554039085e-09),
]


def _arc_error_normalized(angle: float) -> float:  # arc.zig:39-41
    return 2.0 / 27.0 * math.pow(math.sin(angle / 4), 6) / math.pow(math.cos(angle / 4), 2)


def _arc_max_angle_for_tolerance_normalized(tolerance: float) -> float:  # arc.zig:43-74
    for angle, err in _ARC_TABLE:
        if err < tolerance:
            return angle
    angle = 0.0
    for i in range(len(_ARC_TABLE), 1000):
        angle = math.pi / float(i)
        if _arc_error_normalized(angle) <= tolerance:
            break
    return angle


def transformed_circle_major_axis(m: Sequence[float], radius: float) -> float:  # arc.zig:92-262
    a, b, c, d = m[0], m[1], m[2], m[3]
    eps = 0.00390625
    det = a * d - b * c
    if abs(det * det - 1.0) < eps and ((abs(b) < eps and abs(c) < eps) or (abs(a) < eps and abs(d) < eps)):
        return radius
    i = a * a + b * b
    j = c * c + d * d
    f = 0.5 * (i + j)
    g = 0.5 * (i - j)
    h = a * c + b * d
    return radius * math.sqrt(f + math.hypot(g, h))


def _arc_segments_needed(angle: float, radius: float, ctm, tolerance: float) -> int:  # arc.zig:76-82
    major = transformed_circle_major_axis(ctm, radius)
    return int(math.ceil(abs(angle) / _arc_max_angle_for_tolerance_normalized(tolerance / major)))


class Path:
    def __init__(self, transformation: Sequence[float] = IDENTITY, tolerance: float = 0.1):
        self.nodes: List[tuple] = []
        self.initial: Optional[Tuple[float, float]] = None
        self.current: Optional[Tuple[float, float]] = None
        self.transformation = tuple(float(v) for v in transformation)
        self.tolerance = float(tolerance)  # used by arcs (Path.zig:66-68)

    def arc(self, xc, yc, radius, angle1, angle2) -> "Path":
        """Path.arc (Path.zig:345-372): clockwise from angle1 to angle2."""
        a2 = float(angle2)
        while a2 < angle1:
            a2 += math.pi * 2
        self._arc_in_direction(float(xc), float(yc), float(radius), float(angle1), a2, True,
                               max(self.tolerance, 0.001))
        return self

    def arc_negative(self, xc, yc, radius, angle1, angle2) -> "Path":
        """Path.arcNegative (Path.zig:378-405): counter-clockwise."""
        a2 = float(angle2)
        while a2 > angle1:
            a2 -= math.pi * 2
        self._arc_in_direction(float(xc), float(yc), float(radius), a2, float(angle1), False,
                               max(self.tolerance, 0.001))
        return self

    def _arc_line_to(self, x: float, y: float) -> None:  # Path.zig:407-425
        if self.current is not None and self.current[0] == x and self.current[1] == y:
            return
        self.line_to(x, y)

    def _arc_segment(self, xc, yc, radius, a, b) -> None:  # arc.zig:288-310
        r_sin_a, r_cos_a = radius * math.sin(a), radius * math.cos(a)
        r_sin_b, r_cos_b = radius * math.sin(b), radius * math.cos(b)
        h = 4.0 / 3.0 * math.tan((b - a) / 4.0)
        self.curve_to(xc + r_cos_a - h * r_sin_a, yc + r_sin_a + h * r_cos_a,
                      xc + r_cos_b + h * r_sin_b, yc + r_sin_b - h * r_cos_b,
                      xc + r_cos_b, yc + r_sin_b)

    def _arc_in_direction(self, xc, yc, radius, amin, amax, forward: bool, tolerance: float) -> None:
        # arc.zig:323-392
        if not (amax * amax >= 0.0 and amin * amin >= 0.0):  # is_finite
            return
        if amax - amin > 2 * math.pi * _MAX_FULL_CIRCLES:
            amax = math.fmod(amax - amin, 2 * math.pi)
            if amax < 0:
                amax += 2 * math.pi
            amin = math.fmod(amin, 2 * math.pi)
            if amin < 0:
                amin += 2 * math.pi
            amax += amin + 2 * math.pi * _MAX_FULL_CIRCLES
        if amax - amin > math.pi:
            amid = amin + (amax - amin) / 2.0
            if forward:
                self._arc_in_direction(xc, yc, radius, amin, amid, forward, tolerance)
                self._arc_in_direction(xc, yc, radius, amid, amax, forward, tolerance)
            else:
                self._arc_in_direction(xc, yc, radius, amid, amax, forward, tolerance)
                self._arc_in_direction(xc, yc, radius, amin, amid, forward, tolerance)
        elif amax != amin:
            segments = _arc_segments_needed(amax - amin, radius, self.transformation, tolerance)
            step = (amax - amin) / float(segments)
            segments -= 1
            if not forward:
                amin, amax = amax, amin
                step = -step
            self._arc_line_to(xc + radius * math.cos(amin), yc + radius * math.sin(amin))
            for _ in range(max(0, segments)):
                self._arc_segment(xc, yc, radius, amin, amin + step)
                amin += step
            self._arc_segment(xc, yc, radius, amin, amax)
        else:
            self._arc_line_to(xc + radius * math.cos(amin), yc + radius * math.sin(amin))

    def _xf(self, x: float, y: float) -> Tuple[float, float]:
        # Transformation.userToDevice (src/Transformation.zig:194-206)
        ax, by, cx, dy, tx, ty = self.transformation
        x, y = _clamp_i24(x), _clamp_i24(y)
        if self.transformation == IDENTITY:
            return (x, y)
        nx = ax * x + by * y
        ny = cx * x + dy * y
        return (nx + tx, ny + ty)

    def move_to(self, x: float, y: float) -> "Path":
        p = self._xf(x, y)
        if self.nodes and self.nodes[-1][0] == abi.MOVE_TO and self.nodes[-1][1:3] == p:
            return self
        self.nodes.append((abi.MOVE_TO, p[0], p[1], 0.0, 0.0, 0.0, 0.0))
        self.initial = p
        self.current = p
        return self

    def line_to(self, x: float, y: float) -> "Path":
        if self.current is None:
            return self.move_to(x, y)
        p = self._xf(x, y)
        self.nodes.append((abi.LINE_TO, p[0], p[1], 0.0, 0.0, 0.0, 0.0))
        self.current = p
        return self

    def rel_line_to(self, x: float, y: float) -> "Path":
        """Path.relLineTo (Path.zig:187-192): a line to the current point
        (taken back to user space) plus (x, y)."""
        if self.current is None:
            raise ValueError("NoCurrentPoint")
        inv = tf_inverse(self.transformation)
        ux, uy = tf_distance(inv, self.current[0], self.current[1])
        return self.line_to(ux + inv[4] + x, uy + inv[5] + y)

    def curve_to(self, x1, y1, x2, y2, x3, y3) -> "Path":
        if self.current is None:
            raise ValueError("NoCurrentPoint")
        p1, p2, p3 = self._xf(x1, y1), self._xf(x2, y2), self._xf(x3, y3)
        self.nodes.append((abi.CURVE_TO, p1[0], p1[1], p2[0], p2[1], p3[0], p3[1]))
        self.current = p3
        return self

    def close(self) -> "Path":
        if self.current is None:
            return self
        self.nodes.append((abi.CLOSE_PATH, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0))
        ix, iy = self.initial
        self.nodes.append((abi.MOVE_TO, ix, iy, 0.0, 0.0, 0.0, 0.0))
        return self  # the current point stays where it was (Path.zig:467-476)

    def reset(self) -> None:
        self.nodes.clear()
        self.initial = None
        self.current = None

    def to_array(self) -> np.ndarray:
        return nodes_array(self.nodes)


def nodes_array(nodes: Sequence[tuple]) -> np.ndarray:
    arr = np.zeros(len(nodes), dtype=NODE_DTYPE)
    for i, nd in enumerate(nodes):
        arr[i]["tag"] = nd[0]
        arr[i]["p"] = nd[1:7]
    return arr
