"""Path programs: z2d's Path calls recorded for the device path builder.

A PathProgram records the calls a caller would make on z2d's Path
(src/Path.zig:116-479: moveTo, lineTo, curveTo, relMoveTo, relLineTo,
relCurveTo, arc, arcNegative, close, reset, setting the transformation and
the tolerance) and glyph outlines (src/internal/Glyph.zig:483-869).
build_paths runs many programs on the device (z2dgpu_build_paths) and
returns each program's device-space nodes, ready for painter.fill.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

from . import abi
from .types import IDENTITY, NODE_DTYPE


class PathProgram:
    """The calls that build one path, in order."""

    def __init__(self, transformation: Sequence[float] = IDENTITY, tolerance: float = 0.1):
        self.transformation = tuple(float(v) for v in transformation)
        self.tolerance = float(tolerance)
        self.cmds: List[Tuple[int, tuple]] = []
        self.glyph_points: List[tuple] = []   # (x, y, flags) of this program's glyphs
        self.glyph_ends: List[int] = []

    def _add(self, op: int, *v: float) -> "PathProgram":
        self.cmds.append((op, tuple(float(x) for x in v)))
        return self

    def move_to(self, x, y):
        return self._add(abi.PATH_MOVE_TO, x, y)

    def line_to(self, x, y):
        return self._add(abi.PATH_LINE_TO, x, y)

    def curve_to(self, x1, y1, x2, y2, x3, y3):
        return self._add(abi.PATH_CURVE_TO, x1, y1, x2, y2, x3, y3)

    def rel_move_to(self, dx, dy):
        return self._add(abi.PATH_REL_MOVE_TO, dx, dy)

    def rel_line_to(self, dx, dy):
        return self._add(abi.PATH_REL_LINE_TO, dx, dy)

    def rel_curve_to(self, dx1, dy1, dx2, dy2, dx3, dy3):
        return self._add(abi.PATH_REL_CURVE_TO, dx1, dy1, dx2, dy2, dx3, dy3)

    def arc(self, xc, yc, radius, angle1, angle2):
        return self._add(abi.PATH_ARC, xc, yc, radius, angle1, angle2)

    def arc_negative(self, xc, yc, radius, angle1, angle2):
        return self._add(abi.PATH_ARC_NEGATIVE, xc, yc, radius, angle1, angle2)

    def close(self):
        return self._add(abi.PATH_CLOSE)

    def reset(self):
        return self._add(abi.PATH_RESET)

    def set_transformation(self, m: Sequence[float]):
        return self._add(abi.PATH_SET_TRANSFORMATION, *m)

    def set_tolerance(self, t: float):
        return self._add(abi.PATH_SET_TOLERANCE, t)

    def glyph(self, points: Sequence[Tuple[int, int, bool]], contour_ends: Sequence[int], units_per_em: int):
        """A simple glyph's outline (TrueType points in font units, on-curve
        flags, the last point index of each contour), appended with the
        current transformation as Outline.appendToPath does."""
        p0, e0 = len(self.glyph_points), len(self.glyph_ends)
        self.glyph_points.extend((int(x), int(y), 1 if on else 0) for x, y, on in points)
        self.glyph_ends.extend(int(e) for e in contour_ends)
        # offsets are relative to this program's glyph data; pack_programs rebases them
        return self._add(abi.PATH_GLYPH, p0, len(points), e0, len(contour_ends), units_per_em)


class Packed:
    """Programs packed into the C ABI's arrays."""

    def __init__(self, progs, cmds, gpts, gends, n_progs, n_cmds, n_gpts, n_gends):
        self.progs, self.cmds, self.gpts, self.gends = progs, cmds, gpts, gends
        self.n_progs, self.n_cmds, self.n_gpts, self.n_gends = n_progs, n_cmds, n_gpts, n_gends


def pack_programs(programs: Sequence[PathProgram]) -> Packed:
    n_cmds = sum(len(p.cmds) for p in programs)
    n_gpts = sum(len(p.glyph_points) for p in programs)
    n_gends = sum(len(p.glyph_ends) for p in programs)
    progs = (abi.z2d_path_program * max(1, len(programs)))()
    cmds = (abi.z2d_path_cmd * max(1, n_cmds))()
    gpts = (abi.z2d_glyph_point * max(1, n_gpts))()
    gends = (C.c_uint16 * max(1, n_gends))()
    k = gp = ge = 0
    for i, p in enumerate(programs):
        progs[i].cmd_offset = k
        progs[i].n_cmds = len(p.cmds)
        for j in range(6):
            progs[i].transformation[j] = p.transformation[j]
        progs[i].tolerance = p.tolerance
        for op, v in p.cmds:
            cmds[k].op = op
            if op == abi.PATH_GLYPH:
                v = (v[0] + gp, v[1], v[2] + ge, v[3], v[4])
            for j, x in enumerate(v):
                cmds[k].v[j] = x
            k += 1
        for (x, y, f) in p.glyph_points:
            gpts[gp].x, gpts[gp].y, gpts[gp].flags = x, y, f
            gp += 1
        for e in p.glyph_ends:
            gends[ge] = e
            ge += 1
    return Packed(progs, cmds, gpts, gends, len(programs), n_cmds, n_gpts, n_gends)


def unpack_nodes(packed: Packed, call: Callable, cap: Optional[int] = None):
    """Runs `call` (z2dgpu_build_paths / z2doracle_build_paths arguments
    after the context) and splits the nodes per program; retries once with
    the exact size when the first guess was too small."""
    n = packed.n_progs
    offsets = (C.c_uint64 * (n + 1))()
    status = (C.c_int32 * max(1, n))()
    cap = cap if cap is not None else max(64, 4 * packed.n_cmds + 16)
    for _ in range(2):
        out = np.zeros(max(1, cap), dtype=NODE_DTYPE)
        rc = call(packed.progs, n, packed.cmds, packed.n_cmds, packed.gpts, packed.n_gpts, packed.gends,
                  packed.n_gends, out.ctypes.data, cap, offsets, status)
        if rc == abi.ERR_OUT_OF_MEMORY and offsets[n] > cap:
            cap = int(offsets[n])
            continue
        if rc != abi.OK:
            raise RuntimeError(f"build_paths failed with status {rc}")
        nodes = [out[offsets[i]:offsets[i + 1]].copy() for i in range(n)]
        return nodes, [int(status[i]) for i in range(n)]
    raise RuntimeError("build_paths: node count changed between calls")


def build_paths(programs: Sequence[PathProgram], ctx=None):
    """Builds every program on the device: (nodes per program as NODE_DTYPE
    arrays, status per program: 0 or the first error)."""
    from .native import default_context
    c = ctx or default_context()
    packed = pack_programs(programs)
    return unpack_nodes(packed, lambda *a: c.lib.z2dgpu_build_paths(c.handle, *a))
