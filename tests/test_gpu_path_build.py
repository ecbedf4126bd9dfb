"""The device path builder (z2dgpu_build_paths) against the oracle's Path.

Every program's nodes, their count and the program's status must equal the
oracle's restatement of z2d's Path (oracle/z2d_path.cpp) bit for bit:
random programs of every command (absolute and relative points, arcs in
both directions with random radii, angles and tolerances, closes, resets,
transformation and tolerance changes, glyph outlines), the error paths
(NoCurrentPoint, transformations that cannot be inverted, arc angles
beyond the reduction range) and real glyphs from the fixture of the
reference's test font.  A filled result of built paths is compared too.
"""
import json
import math
import os

import numpy as np
import pytest

from backends import GpuBackend
from z2d_gb300 import abi
from z2d_gb300.path_program import PathProgram, build_paths

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()

GLYPHS = os.path.join(os.path.dirname(__file__), "golden", "glyphs_inter_regular.json")


def _tf(rng):
    r = rng.random()
    if r < 0.3:
        return (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    if r < 0.4:
        return (float(rng.uniform(0.5, 3)), 0.0, 0.0, float(rng.uniform(0.5, 3)), *map(float, rng.uniform(-50, 50, 2)))
    if r < 0.45:  # singular: rel* commands fail with InvalidMatrix
        return (1.0, 2.0, 0.5, 1.0, 3.0, 4.0)
    a = rng.uniform(-math.pi, math.pi)
    sx, sy = rng.uniform(0.2, 4, 2)
    sh = rng.uniform(-0.6, 0.6)
    c, s = math.cos(a), math.sin(a)
    return (c * sx, -s * sy + sh, s * sx, c * sy, *map(float, rng.uniform(-400, 400, 2)))


def _random_glyph(rng):
    n_contours = int(rng.integers(1, 4))
    pts, ends = [], []
    for _ in range(n_contours):
        n = int(rng.integers(1, 14))
        for _ in range(n):
            pts.append((int(rng.integers(-800, 2200)), int(rng.integers(-600, 2000)), bool(rng.random() < 0.55)))
        ends.append(len(pts) - 1)
    return pts, ends


def _random_program(rng):
    p = PathProgram(_tf(rng), tolerance=float(rng.choice([0.1, 0.01, 0.3, 1e-4])))
    for _ in range(int(rng.integers(0, 40))):
        r = rng.random()
        x, y = map(float, rng.uniform(-600, 600, 2))
        if r < 0.12:
            p.move_to(x, y)
        elif r < 0.3:
            p.line_to(x, y)
        elif r < 0.4:
            p.curve_to(*map(float, rng.uniform(-600, 600, 4)), x, y)
        elif r < 0.46:
            p.rel_move_to(x / 8, y / 8)
        elif r < 0.52:
            p.rel_line_to(x / 8, y / 8)
        elif r < 0.57:
            p.rel_curve_to(*map(float, rng.uniform(-60, 60, 6)))
        elif r < 0.66:
            p.close()
        elif r < 0.8:
            rad = float(rng.choice([rng.uniform(0.5, 300), 0.0, -20.0]))
            a1, a2 = map(float, rng.uniform(-20, 20, 2))
            (p.arc if rng.random() < 0.5 else p.arc_negative)(x, y, rad, a1, a2)
        elif r < 0.84:
            p.set_transformation(_tf(rng))
        elif r < 0.86:
            p.set_tolerance(float(rng.choice([0.1, 0.05, 2.0])))
        elif r < 0.88:
            p.reset()
        elif r < 0.95:
            pts, ends = _random_glyph(rng)
            p.glyph(pts, ends, int(rng.choice([1000, 2048])))
        elif r < 0.97:
            p.move_to(x, y).move_to(x, y)  # the repeated move_to is dropped
        else:
            p.line_to(float("nan"), 1e30)  # NaN clamps to the upper bound
    return p


def _compare(got, want, what):
    (gn, gs), (wn, ws) = got, want
    assert gs == ws, f"{what}: status {gs} vs {ws}"
    assert len(gn) == len(wn)
    for k, (a, b) in enumerate(zip(gn, wn)):
        assert len(a) == len(b), f"{what} program {k}: {len(a)} nodes vs {len(b)}"
        assert np.array_equal(a["tag"], b["tag"]), f"{what} program {k}: tags differ"
        bad = np.flatnonzero((a["p"].view(np.uint64) != b["p"].view(np.uint64)).any(1))
        assert bad.size == 0, f"{what} program {k}: node {bad[0]} {a[bad[0]]} vs {b[bad[0]]}"


@pytest.mark.parametrize("seed", range(6))
def test_random_programs(oracle, seed):
    rng = np.random.default_rng(500 + seed)
    progs = [_random_program(rng) for _ in range(400)]
    _compare(build_paths(progs), oracle.build_paths(progs), f"seed {seed}")


def test_errors_and_limits(oracle):
    progs = [
        PathProgram().curve_to(1, 2, 3, 4, 5, 6),                                  # NoCurrentPoint
        PathProgram().move_to(1, 1).rel_line_to(2, 2).set_transformation((1, 2, 2, 4, 0, 0)).rel_line_to(1, 1),
        PathProgram().move_to(0, 0).arc(10, 10, 5, 1e7, 1e7 + 1),                  # beyond 2^20 pi/2
        PathProgram().move_to(0, 0).arc(10, 10, 5, 0, 2 * math.pi * 70000),         # full-circle normalisation
        PathProgram().arc(10, 10, 5, 3, -1e5),                                      # many whole turns
        PathProgram().arc_negative(10, 10, 5, -3, 1e5),
        PathProgram().move_to(0, 0).line_to(5, 5).close().rel_line_to(1, 0),       # current point after close
        PathProgram().arc(0, 0, 10, 0.5, 0.5),                                      # empty arc: one line_to
        PathProgram().move_to(1, 1).reset().line_to(2, 2),
    ]
    _compare(build_paths(progs), oracle.build_paths(progs), "errors")


def test_fixture_glyphs(oracle):
    """Simple glyphs of the reference's test font (tests/golden), laid out
    as a line of text under a font-size transformation."""
    with open(GLYPHS) as f:
        fx = json.load(f)
    progs = []
    for size in (12.0, 48.0, 300.0):
        s = size / fx["units_per_em"]
        p = PathProgram()
        x = 10.0
        for g in fx["glyphs"]:
            p.set_transformation((s, 0.0, 0.0, s, x, size * 1.2))
            p.glyph([tuple(q) for q in g["points"]], g["ends"], fx["units_per_em"])
            x += g["advance"] * s
        progs.append(p)
    got, want = build_paths(progs), oracle.build_paths(progs)
    _compare(got, want, "fixture glyphs")
    assert all(st == 0 for st in got[1])
    assert any((n["tag"] == abi.CURVE_TO).any() for n in got[0])


def test_built_paths_fill(gpu, oracle):
    """Nodes built on the device fill the same pixels as the oracle's nodes
    filled by the oracle."""
    from z2d_gb300.surface import Surface
    from z2d_gb300.types import FillOptions, Pattern, Pixel
    rng = np.random.default_rng(77)
    progs = []
    for _ in range(24):
        p = PathProgram(_tf(rng) if rng.random() < 0.5 else (1.0, 0.0, 0.0, 1.0, 0.0, 0.0))
        cx, cy = map(float, rng.uniform(20, 236, 2))
        p.move_to(cx, cy).arc(cx, cy, float(rng.uniform(5, 90)), *map(float, rng.uniform(-6, 6, 2))).close()
        p.move_to(cx + 5, cy).line_to(cx + 40, cy + 30).curve_to(cx, cy + 80, cx - 30, cy, cx - 40, cy - 20).close()
        progs.append(p)
    got_nodes, st = build_paths(progs)
    want_nodes, _ = oracle.build_paths(progs)
    assert all(s == 0 for s in st)
    a, b = Surface.init("rgba", 256, 256), Surface.init("rgba", 256, 256)
    for k, (gn, wn) in enumerate(zip(got_nodes, want_nodes)):
        pat = Pattern.from_pixel(Pixel.rgba(int(20 + k * 9), 80, 200 - k * 5, 230))
        opts = FillOptions(fill_rule="even_odd" if k & 1 else "non_zero")
        assert gpu.fill(a, pat, gn, opts) == abi.OK
        assert oracle.fill(b, pat, wn, opts) == abi.OK
    assert np.array_equal(a.numpy(), b.numpy())
