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


def random_path_batch(rng: np.random.Generator, n: int, w: int, h: int, side_lo: float, side_hi: float,
                      seg_lo: int = 3, seg_hi: int = 64) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """n paths distributed like random_path, generated together: returns the
    concatenated node array and each path's node offset and count.  Each path
    is move_to + segments + close_path + move_to(initial)."""
    side = rng.uniform(side_lo, side_hi, n)
    x0 = rng.uniform(0.0, 1.0, n) * np.maximum(0.0, w - side)
    y0 = rng.uniform(0.0, 1.0, n) * np.maximum(0.0, h - side)
    nseg = rng.integers(seg_lo, seg_hi + 1, n)
    count = nseg + 3
    off = np.zeros(n, np.int64)
    np.cumsum(count[:-1], out=off[1:])
    total = int(count.sum())
    nodes = np.zeros(total, NODE_DTYPE)
    pid = np.repeat(np.arange(n), count)
    k = np.arange(total) - off[pid]          # position inside the path
    pts = rng.uniform(0.0, 1.0, (total, 6)) * side[pid, None]
    pts[:, 0::2] += x0[pid, None]
    pts[:, 1::2] += y0[pid, None]
    curve = rng.random(total) >= 0.5
    tag = np.where(curve, abi.CURVE_TO, abi.LINE_TO).astype(np.int32)
    tag[k == 0] = abi.MOVE_TO
    last = off + count - 1
    tag[last - 1] = abi.CLOSE_PATH
    tag[last] = abi.MOVE_TO
    pts[tag != abi.CURVE_TO, 2:] = 0.0
    pts[tag == abi.CLOSE_PATH] = 0.0
    pts[last, :2] = pts[off, :2]              # the move_to after close returns to the start
    nodes["tag"] = tag
    nodes["p"] = pts
    return nodes, off, count


def batched_jobs(seed: int, n_jobs: int, side_lo: int = 16, side_hi: int = 2048, paths_lo: int = 1,
                 paths_hi: int = 200):
    """The batched-jobs configuration: RGBA jobs whose sides are
    log-uniform in [side_lo, side_hi], each with paths_lo..paths_hi random
    closed paths generated like the large plain workload (3-64 segments, half
    lines and half cubics, rule alternating, premultiplied pixel sources with
    alpha U[32,255], src_over) with path boxes scaled to the job (side
    U[side/64, side/2]).  Stroked paths are not included.  Returns, per job,
    (width, height, nodes, node offsets, node counts, pixels (n x 4 RGBA),
    rules)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_jobs):
        w = int(round(math.exp(rng.uniform(math.log(side_lo), math.log(side_hi)))))
        h = int(round(math.exp(rng.uniform(math.log(side_lo), math.log(side_hi)))))
        n = int(rng.integers(paths_lo, paths_hi + 1))
        s = min(w, h)
        nodes, off, cnt = random_path_batch(rng, n, w, h, max(2.0, s / 64), max(4.0, s / 2))
        a = rng.integers(32, 256, n)
        rgb = (rng.random((n, 3)) * (a[:, None] + 1)).astype(np.int64)
        px = np.concatenate([np.minimum(rgb, a[:, None]), a[:, None]], 1).astype(np.uint8)
        rules = np.where(np.arange(n) % 2 == 0, abi.FILL_EVEN_ODD, abi.FILL_NON_ZERO).astype(np.int32)
        out.append((w, h, nodes, off, cnt, px, rules))
    return out


def job_fills(job) -> List[Tuple[Pattern, np.ndarray, FillOptions]]:
    """The (pattern, nodes, options) list of one batched_jobs entry."""
    w, h, nodes, off, cnt, px, rules = job
    names = {abi.FILL_EVEN_ODD: "even_odd", abi.FILL_NON_ZERO: "non_zero"}
    return [(Pattern.from_pixel(Pixel.rgba(*map(int, px[i]))), nodes[off[i]:off[i] + cnt[i]],
             FillOptions(fill_rule=names[int(rules[i])])) for i in range(len(off))]


def glyph_path(rng: np.random.Generator, box: float = 64.0, cubics_lo: int = 20, cubics_hi: int = 200) -> np.ndarray:
    """A glyph-like closed outline: 20-200 cubic Beziers whose control points
    wander around an ellipse inside a box x box square (several subpaths
    for counters are not modelled)."""
    n = int(rng.integers(cubics_lo, cubics_hi + 1))
    t = np.sort(rng.uniform(0.0, 2 * math.pi, n))
    rx, ry = box * rng.uniform(0.25, 0.45), box * rng.uniform(0.25, 0.45)
    cx, cy = box / 2, box / 2
    wob = rng.uniform(0.6, 1.0, n)
    ends = np.stack([cx + rx * wob * np.cos(t), cy + ry * wob * np.sin(t)], 1)
    pts = [(abi.MOVE_TO, float(ends[-1, 0]), float(ends[-1, 1]))]
    prev = ends[-1]
    for k in range(n):
        c1 = prev + rng.uniform(-box / 8, box / 8, 2)
        c2 = ends[k] + rng.uniform(-box / 8, box / 8, 2)
        pts.append((abi.CURVE_TO, *map(float, np.clip(c1, 0, box)), *map(float, np.clip(c2, 0, box)),
                    float(ends[k, 0]), float(ends[k, 1])))
        prev = ends[k]
    return _path_nodes(pts)
