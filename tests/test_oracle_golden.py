"""Pins the CPU oracle to z2d itself: the reference's golden PNGs for the
fill/compositor spec scenes and its compositor known-answer tests."""
import json
import os

import numpy as np
import pytest

from pngio import export_pixels, golden_pixels, golden_scanlines
from backends import StrokeOracle
from scenes import AA_SUFFIX, COMPOSITOR_SCENES, EXPORT_SCENES, FILL_SCENES, STROKE_SCENES
from z2d_gb300.types import Color, Pixel

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("aa", list(AA_SUFFIX))
@pytest.mark.parametrize("name", list(FILL_SCENES))
def test_fill_scene_matches_golden(oracle, golden_dir, name, aa):
    path = os.path.join(golden_dir, name + AA_SUFFIX[aa] + ".png")
    if not os.path.exists(path):  # MSAA falls back to the SSAA golden (spec/main_spec.zig:786-800)
        path = os.path.join(golden_dir, name + "_smooth.png")
    got = export_pixels(FILL_SCENES[name](oracle, aa))
    exp = golden_pixels(path)
    assert got.shape == exp.shape
    assert int((got != exp).any(-1).sum()) == 0


@pytest.mark.parametrize("aa", list(AA_SUFFIX))
@pytest.mark.parametrize("name", list(STROKE_SCENES))
def test_stroke_scene_matches_golden(oracle, golden_dir, name, aa):
    """Pins the oracle's own stroke tessellation (oracle/z2d_stroke.cpp) to
    z2d: its polygons, rasterised by the oracle, reproduce the golden PNGs."""
    path = os.path.join(golden_dir, name + AA_SUFFIX[aa] + ".png")
    if not os.path.exists(path):
        path = os.path.join(golden_dir, name + "_smooth.png")
    got = export_pixels(STROKE_SCENES[name](StrokeOracle(oracle), aa))
    exp = golden_pixels(path)
    assert got.shape == exp.shape
    assert int((got != exp).any(-1).sum()) == 0


@pytest.mark.parametrize("name", list(COMPOSITOR_SCENES))
def test_compositor_scene_matches_golden(oracle, golden_dir, name):
    got = export_pixels(COMPOSITOR_SCENES[name](oracle))
    exp = golden_pixels(os.path.join(golden_dir, name + ".png"))
    assert got.shape == exp.shape
    assert np.array_equal(got, exp)


def _kats():
    with open(os.path.join(HERE, "golden", "compositor_kats.json")) as f:
        d = json.load(f)
    return [(prec, i, c) for prec in ("integer", "float") for i, c in enumerate(d[prec])]


@pytest.mark.parametrize("prec,idx,case", _kats(), ids=lambda v: str(v) if not isinstance(v, dict) else v["op"])
def test_compositor_kat(oracle, prec, idx, case):
    bg = oracle.pixel_from_color(Color.rgb(*case["bg"]))
    fg = oracle.pixel_from_color(Color.rgb(*case["fg"]))
    r = oracle.run_pixel(prec, Pixel(bg.format, bg.r, bg.g, bg.b, bg.a),
                         Pixel(fg.format, fg.r, fg.g, fg.b, fg.a), case["op"])
    assert [r.r, r.g, r.b, r.a] == case["expected"]


@pytest.mark.parametrize("aa", list(AA_SUFFIX))
@pytest.mark.parametrize("name", sorted(list(FILL_SCENES) + list(STROKE_SCENES)))
def test_png_scanlines_match_golden(oracle, golden_dir, name, aa):
    """The exporter's uncompressed image data (export_png.zig:153-372) of the
    oracle's render equals the golden PNG's, byte for byte."""
    path = os.path.join(golden_dir, name + AA_SUFFIX[aa] + ".png")
    if not os.path.exists(path):
        path = os.path.join(golden_dir, name + "_smooth.png")
    scene = FILL_SCENES.get(name) or STROKE_SCENES[name]
    assert oracle.png_scanlines(scene(StrokeOracle(oracle), aa)) == golden_scanlines(path)


@pytest.mark.parametrize("name", sorted(list(COMPOSITOR_SCENES) + list(EXPORT_SCENES)))
def test_png_scanlines_match_golden_compositor(oracle, golden_dir, name):
    scene, profile = EXPORT_SCENES.get(name, (COMPOSITOR_SCENES.get(name), None))
    assert oracle.png_scanlines(scene(StrokeOracle(oracle)), profile) == \
        golden_scanlines(os.path.join(golden_dir, name + ".png"))


def _math_kats(kind):
    with open(os.path.join(HERE, "golden", "math_kats.json")) as f:
        return json.load(f)[kind]


@pytest.mark.parametrize("case", _math_kats("pow_f32"), ids=lambda c: f"{c['exponent']}-{c['x']}")
def test_pow_f32_kat(oracle, case):
    """std.math.pow(f32) as z2d computes it: the exact values z2d's own
    SRGB.removeGamma / applyGamma tests expect (src/color.zig:1030-1056,
    compared there with expectEqualDeep)."""
    g = np.float32(2.2)
    y = g if case["exponent"] == "gamma" else np.float32(1.0) / g
    got = np.float32(oracle.pow_f32(float(case["x"]), float(y)))
    assert got == np.float32(case["expected"])


def test_pow_f32_kats_reject_rounded_double_pow():
    """The KATs discriminate: pow evaluated in double and rounded once (the
    host libm) misses some of them, so the exact restatement is needed."""
    g = np.float32(2.2)
    misses = 0
    for case in _math_kats("pow_f32"):
        y = g if case["exponent"] == "gamma" else np.float32(1.0) / g
        misses += np.float32(float(case["x"]) ** float(y)) != np.float32(case["expected"])
    assert misses > 0


@pytest.mark.parametrize("case", _math_kats("conic_offset"), ids=lambda c: c["name"])
def test_conic_offset_kat(oracle, case):
    """Conic.getOffset (std.math.atan2(f64), src/gradient.zig:731-741):
    z2d's exact expected offsets (src/gradient.zig:1702-1766)."""
    from z2d_gb300.types import Gradient
    g = Gradient.conic(case["center_x"], case["center_y"], case["angle"])
    if case["scale"]:
        g.set_transformation((case["scale"][0], 0.0, 0.0, case["scale"][1], 0.0, 0.0))
    assert np.float32(oracle.gradient_offset(g, case["x"], case["y"])) == np.float32(case["expected"])


def test_atan2_accuracy(oracle):
    """The atan2 restatement stays within one ulp of the correctly rounded
    value over all quadrants (a check on its constants and reduction)."""
    rng = np.random.default_rng(5)
    ys = np.concatenate([rng.normal(0, 100, 4000), rng.uniform(-1e-3, 1e-3, 500), [0.0, -0.0, 1.0, -1.0]])
    xs = np.concatenate([rng.normal(0, 100, 4000), rng.uniform(-1e3, 1e3, 500), [1.0, -1.0, 0.0, 2.0]])
    for y, x in zip(ys, xs):
        got = oracle.atan2(float(y), float(x))
        ref = np.arctan2(y, x)
        assert abs(got - ref) <= np.spacing(abs(ref)) + 1e-300


def _random_strokes(n, seed):
    from z2d_gb300.types import StrokeOptions
    from z2d_gb300.workloads import random_path
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nodes = random_path(rng, 300, 200, 10, 250, 3, 20)
        dashed = i % 3 == 0
        tf = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0) if i % 4 else (1.5, 0.3, -0.2, 0.8, 4.0, -3.0)
        so = StrokeOptions(line_width=float(rng.uniform(0.5, 20)), line_join=("miter", "round", "bevel")[i % 3],
                           line_cap=("butt", "round", "square")[(i // 3) % 3],
                           dashes=tuple(rng.uniform(0, 40, int(rng.integers(2, 7)))) if dashed else (),
                           dash_offset=float(rng.uniform(-20, 20)) if dashed else 0.0, hairline=(i % 17 == 0),
                           transformation=tf, tolerance=float(rng.choice([0.05, 0.1, 0.5])))
        out.append((nodes, so))
    return out


def test_host_stroke_builder_matches_oracle_stroker(oracle):
    """The library's host stroke builder (z2dgpu_stroke_contours, which
    builds dashed strokes for z2dgpu_draw_jobs) and the oracle's independent
    restatement produce bit-identical polygons on random solid and dashed
    strokes of every join and cap, through plain and skewed transformations,
    and identical hairline polylines (the dasher's empty polylines, which
    draw nothing, aside)."""
    from z2d_gb300 import painter
    for i, (nodes, so) in enumerate(_random_strokes(300, 21)):
        a, sa = painter.stroke_contours(nodes, so, "rgba")
        b, sb = oracle.stroke_contours(nodes, so, "rgba")
        if so.hairline:
            b = [c for c in b if len(c)]
        assert sa == sb and len(a) == len(b), f"stroke {i}: {len(a)} vs {len(b)} contours"
        for k, (x, y) in enumerate(zip(a, b)):
            assert x.shape == y.shape and np.array_equal(x, y), f"stroke {i} contour {k}"
