"""Seeded synthetic workloads with the shapes of the benchmark configurations.

 * star_300():        a 300x300 RGBA surface and one closed 5-point star
                      (outer radius 140, inner 56, centred at (150,150),
                      first point at -90 deg), opaque red, src_over.
 * random_fills():    N random closed paths of 3-64 segments (half lines,
                      half cubic Beziers) whose control points are uniform in
                      an axis-aligned box of side U[16,1024] placed uniformly
                      on the surface; fill rule alternates even-odd/non-zero;
                      premultiplied RGBA pixel sources with alpha U[32,255].
 * premultiplied_background(): uniform premultiplied RGBA pixels.
All randomness comes from numpy's PCG64 with an explicit seed.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from . import abi
from .types import NODE_DTYPE, FillOptions, Pattern, Pixel


def _path_nodes(points: List[tuple]) -> np.ndarray:
    """move_to + segments + close_path + move_to(initial), as Path.close emits."""
    arr = np.zeros(len(points) + 2, NODE_DTYPE)
    for i, p in enumerate(points):
        arr[i]["tag"] = p[0]
        arr[i]["p"][: len(p) - 1] = p[1:]
    arr[len(points)]["tag"] = abi.CLOSE_PATH
    arr[len(points) + 1]["tag"] = abi.MOVE_TO
    arr[len(points) + 1]["p"][:2] = points[0][1:3]
    return arr


def star_300() -> Tuple[int, int, np.ndarray, Pattern, FillOptions]:
    pts = []
    for k in range(10):
        r = 140.0 if k % 2 == 0 else 56.0
        a = math.radians(-90.0 + 36.0 * k)
        x, y = 150.0 + r * math.cos(a), 150.0 + r * math.sin(a)
        pts.append((abi.MOVE_TO if k == 0 else abi.LINE_TO, x, y))
    return 300, 300, _path_nodes(pts), Pattern.from_pixel(Pixel.rgba(255, 0, 0, 255)), FillOptions()


def premultiplied_background(rng: np.random.Generator, w: int, h: int) -> np.ndarray:
    a = rng.integers(0, 256, size=(h * w,), dtype=np.uint16)
    rgb = (rng.random((h * w, 3)) * (a[:, None] + 1)).astype(np.uint16)
    rgb = np.minimum(rgb, a[:, None])
    out = np.empty((h * w, 4), np.uint8)
    out[:, :3] = rgb
    out[:, 3] = a
    return out.reshape(-1)


def random_path(rng: np.random.Generator, w: int, h: int, side_lo=16.0, side_hi=1024.0,
                seg_lo=3, seg_hi=64) -> np.ndarray:
    side = rng.uniform(side_lo, side_hi)
    x0 = rng.uniform(0.0, max(0.0, w - side))
    y0 = rng.uniform(0.0, max(0.0, h - side))
    n = int(rng.integers(seg_lo, seg_hi + 1))

    def pt():
        return (x0 + rng.uniform(0.0, side), y0 + rng.uniform(0.0, side))

    sx, sy = pt()
    pts = [(abi.MOVE_TO, sx, sy)]
    for _ in range(n):
        if rng.random() < 0.5:
            x, y = pt()
            pts.append((abi.LINE_TO, x, y))
        else:
            (ax, ay), (bx, by), (cx, cy) = pt(), pt(), pt()
            pts.append((abi.CURVE_TO, ax, ay, bx, by, cx, cy))
    return _path_nodes(pts)


def random_premultiplied_pixel(rng: np.random.Generator) -> Pixel:
    a = int(rng.integers(32, 256))
    r, g, b = (int(rng.integers(0, a + 1)) for _ in range(3))
    return Pixel.rgba(r, g, b, a)


def random_fills(seed: int, n: int, w: int, h: int, **kw) -> List[Tuple[Pattern, np.ndarray, FillOptions]]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nodes = random_path(rng, w, h, **kw)
        px = random_premultiplied_pixel(rng)
        rule = "even_odd" if i % 2 == 0 else "non_zero"
        out.append((Pattern.from_pixel(px), nodes, FillOptions(fill_rule=rule)))
    return out


def fill_box_pixels(nodes: np.ndarray, w: int, h: int, scale: float = 4.0) -> int:
    """Pixels of multisample.run's clamped draw box (multisample.zig:46-78)
    for a path of line segments and curve control points (the control-point
    hull bounds the flattened curve)."""
    pts = []
    for nd in nodes:
        t = nd["tag"]
        if t in (abi.MOVE_TO, abi.LINE_TO):
            pts.append(nd["p"][:2])
        elif t == abi.CURVE_TO:
            pts.extend([nd["p"][0:2], nd["p"][2:4], nd["p"][4:6]])
    p = np.array(pts) * scale
    el, et = p[:, 0].min(), p[:, 1].min()
    er, eb = p[:, 0].max(), p[:, 1].max()
    sy = min(max(int(math.floor(et / scale)), 0), h - 1)
    ey = min(max(int(math.ceil(eb / scale)), sy), h - 1)
    sx = min(max(int(math.floor(el / scale)), 0), w - 1)
    ex = min(max(int(math.ceil(er / scale)), sx), w)
    return (ey - sy + 1) * (ex - sx)
