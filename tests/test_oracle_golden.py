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
    """Pins the host stroke builder (z2dgpu_stroke_contours) to z2d: its
    polygons, rasterised by the oracle, reproduce the golden PNGs."""
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
