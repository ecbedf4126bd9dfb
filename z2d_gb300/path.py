"""Path builder producing the node arrays painter.fill consumes.

Mirrors z2d's Path (src/Path.zig:116-262, 447-477): coordinates are clamped
to the i24 range (clampI24, :570), transformed by the current matrix at
insertion, a repeated move_to to the same point is dropped, and close()
appends close_path plus a move_to back to the subpath's initial point.
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import abi
from .types import IDENTITY, NODE_DTYPE

_I24_MIN, _I24_MAX = -(1 << 23), (1 << 23) - 1


def _clamp_i24(v: float) -> float:
    return min(max(float(v), _I24_MIN), _I24_MAX)


class Path:
    def __init__(self, transformation: Sequence[float] = IDENTITY):
        self.nodes: List[tuple] = []
        self.initial: Optional[Tuple[float, float]] = None
        self.current: Optional[Tuple[float, float]] = None
        self.transformation = tuple(float(v) for v in transformation)

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
        self.current = self.initial
        return self

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
