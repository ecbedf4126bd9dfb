"""PNG export on the GPU (z2dgpu_png_encode / z2dgpu_png_scanlines)
against the oracle's restatement of the exporter, whose image data is
pinned to the golden PNGs byte for byte (test_oracle_golden.py)."""
import zlib

import numpy as np
import pytest

from backends import GpuBackend, StrokeOracle
from pngio import png_chunks
from scenes import EXPORT_SCENES, FILL_SCENES, STROKE_SCENES
from z2d_gb300 import abi, png
from z2d_gb300.surface import Surface

pytestmark = pytest.mark.gpu

FORMATS = ["rgba", "argb", "rgb", "xrgb", "alpha8", "alpha4", "alpha2", "alpha1"]


def _random_surface(fmt, w, h, seed):
    rng = np.random.default_rng(seed)
    s = Surface.init(fmt, w, h)
    d = rng.integers(0, 256, size=s.data.size, dtype=np.uint8)
    if fmt in ("rgba", "argb"):  # premultiplied: colour <= alpha, some zero alphas
        px = d.reshape(-1, 4)
        a_idx = 3
        px[:, a_idx] = np.where(rng.random(len(px)) < 0.1, 0, px[:, a_idx])
        for c in range(3):
            px[:, c] = (px[:, c].astype(np.uint32) * px[:, a_idx] // 255).astype(np.uint8)
    s.data[:] = d
    return s


@pytest.mark.parametrize("profile", [None, "linear", "srgb"])
@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (33, 17), (257, 5)])
def test_scanlines_match_oracle(oracle, fmt, w, h, profile):
    s = _random_surface(fmt, w, h, w * 131 + h + len(fmt))
    assert png.scanlines(s, profile) == oracle.png_scanlines(s, profile)
    d = s.to_device("cuda")  # device-resident surfaces export the same
    assert png.scanlines(d, profile) == oracle.png_scanlines(s, profile)


@pytest.mark.parametrize("fmt", FORMATS)
def test_png_file_structure(oracle, fmt):
    """Signature, IHDR (depth / colour type of export_png.zig:97-131), gAMA
    for a profile, CRCs, and IDAT decoding to the exporter's image data."""
    s = _random_surface(fmt, 45, 21, 9)
    for profile, gamma in ((None, None), ("linear", 100000), ("srgb", 45454)):
        data = png.encode(s, profile)
        chunks = png_chunks(data)
        types = [t for t, _ in chunks]
        assert types[0] == b"IHDR" and types[-1] == b"IEND"
        ihdr = chunks[0][1]
        depth, ctype = ihdr[8], ihdr[9]
        assert int.from_bytes(ihdr[0:4], "big") == 45 and int.from_bytes(ihdr[4:8], "big") == 21
        assert depth == {"alpha4": 4, "alpha2": 2, "alpha1": 1}.get(fmt, 8)
        assert ctype == {"rgba": 6, "argb": 6, "rgb": 2, "xrgb": 2}.get(fmt, 0)
        gama = [b for t, b in chunks if t == b"gAMA"]
        assert (int.from_bytes(gama[0], "big") if gama else None) == gamma
        raw = zlib.decompress(b"".join(b for t, b in chunks if t == b"IDAT"))
        assert raw == oracle.png_scanlines(s, profile)


@pytest.mark.parametrize("name", ["003_fill_triangle", "033_fill_zig_mark", "051_fill_triangle_alpha1_gray",
                                  "070_compositor_ops", "081_stroke_hairline", "058_stroke_misc_dashes"])
def test_scene_export(oracle, name):
    """A scene drawn and exported on the GPU equals the oracle's drawing
    exported by the oracle (the latter equals the golden's image data)."""
    scene = FILL_SCENES.get(name) or STROKE_SCENES[name]
    assert png.scanlines(scene(GpuBackend(), "default")) == oracle.png_scanlines(scene(StrokeOracle(oracle), "default"))


@pytest.mark.parametrize("name", list(EXPORT_SCENES))
def test_gamma_scene_export(oracle, name):
    scene, profile = EXPORT_SCENES[name]
    assert png.scanlines(scene(GpuBackend()), profile) == oracle.png_scanlines(scene(StrokeOracle(oracle)), profile)
