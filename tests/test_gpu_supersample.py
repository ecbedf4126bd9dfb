"""Supersample anti-aliasing (supersample.run, src/internal/raster/supersample.zig:17-185)
on the GPU against the oracle.

The GPU draws a supersample fill as a coverage count per pixel (the 4x4
samples the downsampled mask averages) followed by the batch
[dst_in(pattern, mask), op] over the whole composite region, so these cases
cover: every pixel format the mask can take (alpha8, or alpha4/2 for those
surfaces), bounded and unbounded operators, integer and float precision,
gradient and dither sources, regions clipped by the surface edges, the
too-small mask that skips the downsample, unbalanced rows (k_exact), and
batches that mix the three anti-aliasing modes.
"""
import numpy as np
import pytest

from backends import GpuBackend
from z2d_gb300 import abi, painter
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, FillOptions, Gradient, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background, random_fills, random_path

pytestmark = pytest.mark.gpu

FLOAT_TOL = 0  # gradients and float operators: bit-exact (Zig's pow/atan2 on both sides)
SS = "supersample_4x"
M, L, Q, C = abi.MOVE_TO, abi.LINE_TO, abi.CURVE_TO, abi.CLOSE_PATH


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()


def _bg(fmt, w, h, seed):
    rng = np.random.default_rng(seed)
    s = Surface.init(fmt, w, h)
    if fmt in ("rgba", "argb"):
        s.data[:] = premultiplied_background(rng, w, h)
    elif fmt in ("rgb", "xrgb"):
        d = rng.integers(0, 256, size=s.data.size, dtype=np.uint8)
        d.reshape(-1, 4)[:, 3] = 0
        s.data[:] = d
    else:
        s.data[:] = rng.integers(0, 256, size=s.data.size, dtype=np.uint8)
    return s


def _cmp(a, b, tol, what):
    x = a.numpy().astype(np.int16)
    y = b.numpy().astype(np.int16)
    d = np.abs(x - y)
    assert int(d.max(initial=0)) <= tol, f"{what}: {int((d > 0).sum())} bytes differ (max {int(d.max())})"


def _both(gpu, oracle, fmt, w, h, seed, draws):
    a, b = _bg(fmt, w, h, seed), _bg(fmt, w, h, seed)
    for pat, nodes, opts in draws:
        assert gpu.fill(a, pat, nodes, opts) == abi.OK
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    return a, b


@pytest.mark.parametrize("fmt", ["rgba", "argb", "rgb", "xrgb", "alpha8", "alpha4", "alpha2"])
def test_supersample_pixel_src_over(gpu, oracle, fmt):
    w, h = 173, 131
    fills = random_fills(seed=17, n=12, w=w, h=h, side_lo=4, side_hi=160, seg_lo=3, seg_hi=24)
    for _, _, opts in fills:
        opts.anti_aliasing = SS
    a, b = _both(gpu, oracle, fmt, w, h, 3, fills)
    _cmp(a, b, 0, fmt)


@pytest.mark.parametrize("precision", ["integer", "float"])
@pytest.mark.parametrize("op", abi.OPERATORS)
def test_supersample_operators(gpu, oracle, op, precision):
    w, h = 97, 83
    fills = random_fills(seed=abi.OP[op] + 300, n=3, w=w, h=h, side_lo=10, side_hi=90, seg_lo=3, seg_hi=12)
    for _, _, opts in fills:
        opts.anti_aliasing = SS
        opts.operator = op
        opts.precision = precision
    a, b = _both(gpu, oracle, "rgba", w, h, 5, fills)
    float_path = precision == "float" or op in abi.FLOAT_ONLY_OPS
    _cmp(a, b, FLOAT_TOL if float_path else 0, f"{op}/{precision}")


@pytest.mark.parametrize("fmt", ["alpha8", "alpha4", "alpha2"])
@pytest.mark.parametrize("op", ["src_over", "src_in", "dst_out", "xor", "clear"])
def test_supersample_alpha_formats(gpu, oracle, fmt, op):
    w, h = 61, 45
    fills = random_fills(seed=abi.OP[op] + 400, n=3, w=w, h=h, side_lo=6, side_hi=60, seg_lo=3, seg_hi=10)
    for _, _, opts in fills:
        opts.anti_aliasing = SS
        opts.operator = op
    a, b = _both(gpu, oracle, fmt, w, h, 6, fills)
    _cmp(a, b, 0, f"{fmt}/{op}")


@pytest.mark.parametrize("source", ["linear", "radial", "conic", "bayer", "blue_noise"])
@pytest.mark.parametrize("precision", ["integer", "float"])
def test_supersample_gradients(gpu, oracle, source, precision):
    g = {"linear": Gradient.linear(5, 7, 110, 80), "radial": Gradient.radial(60, 45, 5, 55, 40, 70),
         "conic": Gradient.conic(60, 45, 0.7), "bayer": Gradient.linear(0, 0, 120, 90, method="srgb"),
         "blue_noise": Gradient.radial(30, 30, 0, 60, 45, 80, method="hsl")}[source]
    g.add_stop(0.0, Color.rgb(1, 0, 0, 0.9))
    g.add_stop(0.4, Color.rgb(0, 1, 0.2, 0.5))
    g.add_stop(1.0, Color.srgb(0.1, 0.2, 0.9, 0.75))
    pat = Pattern.dither(source, g, 8) if source in ("bayer", "blue_noise") else Pattern.from_gradient(g)
    rng = np.random.default_rng(21)
    w, h = 120, 90
    draws = []
    for i in range(3):
        opts = FillOptions(precision=precision, anti_aliasing=SS, operator="src_over" if i != 1 else "multiply")
        draws.append((pat, random_path(rng, w, h, 20, 110, 3, 10), opts))
    a, b = _both(gpu, oracle, "rgba", w, h, 7, draws)
    _cmp(a, b, FLOAT_TOL, f"{source}/{precision}")


def _tri(x0, y0, x1, y1, x2, y2):
    return [(M, x0, y0, 0, 0, 0, 0), (L, x1, y1, 0, 0, 0, 0), (L, x2, y2, 0, 0, 0, 0), (C, 0, 0, 0, 0, 0, 0)]


EDGE_CASES = {
    # the polygon ends exactly at x = 0 (or y = 0): a 1-sample-wide mask that
    # is never downsampled and stays empty, composited over a 1-pixel column
    "right_extent_zero": _tri(-30, 5, 0, 20, -10, 40),
    "bottom_extent_zero": _tri(5, -30, 20, 0, 40, -10),
    "both_extents_zero": _tri(-30, -30, 0, -10, -10, 0),
    # regions clipped by every surface edge
    "overhang_left_top": _tri(-20, -15, 30, 10, 5, 25),
    "overhang_right_bottom": _tri(50, 40, 90, 70, 70, 95),
    "covers_surface": _tri(-100, -100, 300, -50, -50, 300),
    # sub-pixel and one-pixel shapes
    "tiny": _tri(10.2, 10.1, 10.7, 10.3, 10.4, 10.9),
    "one_pixel": _tri(20, 20, 21, 20, 21, 21),
    # a 2-point closed subpath leaves one unmatched edge (k_exact)
    "unbalanced": _tri(5, 5, 60, 12, 30, 50) + [(M, 40, 2, 0, 0, 0, 0), (L, 20, 58, 0, 0, 0, 0), (C, 0, 0, 0, 0, 0, 0)],
    "curve": [(M, 5, 30, 0, 0, 0, 0), (Q, 20, -10, 50, 70, 70, 25), (L, 60, 55, 0, 0, 0, 0), (C, 0, 0, 0, 0, 0, 0)],
}


@pytest.mark.parametrize("op", ["src_over", "clear", "src_in", "dst_atop", "multiply"])
@pytest.mark.parametrize("case", list(EDGE_CASES))
@pytest.mark.parametrize("fmt", ["rgba", "alpha4"])
def test_supersample_edge_cases(gpu, oracle, case, op, fmt):
    w, h = 73, 61
    pat = Pattern.from_pixel(Pixel.rgba(90, 40, 160, 200))
    for rule in ("non_zero", "even_odd"):
        opts = FillOptions(anti_aliasing=SS, operator=op, fill_rule=rule)
        a, b = _both(gpu, oracle, fmt, w, h, 9, [(pat, EDGE_CASES[case], opts)])
        _cmp(a, b, 0, f"{case}/{op}/{rule}/{fmt}")


def test_supersample_batch_mixed_modes(oracle):
    w, h = 300, 220
    fills = random_fills(seed=31, n=90, w=w, h=h, side_lo=6, side_hi=200, seg_lo=3, seg_hi=30)
    modes = ["supersample_4x", "default", "none"]
    ops = ["src_over", "src_over", "multiply", "src_in", "screen", "clear"]
    for i, (_, _, opts) in enumerate(fills):
        opts.anti_aliasing = modes[i % 3]
        opts.operator = ops[(i // 3) % len(ops)]
    a, b = _bg("rgba", w, h, 11), _bg("rgba", w, h, 11)
    painter.fill_batch(a, fills)
    for pat, nodes, opts in fills:
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, "mixed batch")
