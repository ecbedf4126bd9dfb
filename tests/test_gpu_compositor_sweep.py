"""The compositor configuration checked cell by cell against the oracle.

The sweep is z2d's mask batch [dst_in(dst = source, src = alpha8 mask), op]
(supersample.zig:171-184 through SurfaceCompositor.run,
compositor.zig:302-440) on whole surfaces whose size takes the fused
kernels (a pixel count divisible by 16 and 16-byte aligned rows of bytes):
every format x every operator x both precisions with a pixel source, and
every gradient kind x interpolation method x dither mode with the source in
the batch.  A larger case repeats a few cells at 1024 x 1024.  Every cell is
bit-exact; the count of differing pixels is in the failure message.
"""
import zlib

import numpy as np
import pytest

from backends import GpuBackend
from z2d_gb300 import abi
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, Gradient, Operation, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background

pytestmark = pytest.mark.gpu

FORMATS = ["rgba", "argb", "rgb", "xrgb", "alpha8", "alpha4", "alpha2", "alpha1"]
W, H = 256, 96  # 24576 px: whole 16-pixel items in every format


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()


def _surface(fmt, w, h, seed):
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


def _mask(w, h, seed):
    m = Surface.init("alpha8", w, h)
    m.data[:] = np.random.default_rng(seed).integers(0, 256, size=m.data.size, dtype=np.uint8)
    return m


def _pixel_diff(a, b, fmt):
    x, y = a.numpy(), b.numpy()
    if abi.FORMAT_NAMES.index(fmt) <= abi.FORMAT_RGBA:
        return int((x.reshape(-1, 4) != y.reshape(-1, 4)).any(1).sum())
    return int((x != y).sum())  # bytes of packed pixels


def _check(gpu, oracle, fmt, ops, precision, w=W, h=H, seed=0, what=""):
    a, b = _surface(fmt, w, h, seed), _surface(fmt, w, h, seed)
    assert gpu.composite(a, 0, 0, ops, precision) == abi.OK
    assert oracle.composite(b, 0, 0, ops, precision) == abi.OK
    n = _pixel_diff(a, b, fmt)
    assert n == 0, f"{what}: {n} differing pixels"


@pytest.mark.parametrize("precision", ["integer", "float"])
@pytest.mark.parametrize("op", abi.OPERATORS)
@pytest.mark.parametrize("fmt", FORMATS)
def test_mask_batch_pixel_source(gpu, oracle, fmt, op, precision):
    src = Pattern.from_pixel(Pixel.rgba(90, 40, 160, 200))
    ops = [Operation("dst_in", dst=src, src=_mask(W, H, abi.OP[op])), Operation(op)]
    _check(gpu, oracle, fmt, ops, precision, seed=abi.OP[op] + 7, what=f"{fmt}/{op}/{precision}")


def _gradient(kind, method, n_stops, seed, k=1.0):
    """A gradient over a 256 x 96 surface (k scales its geometry)."""
    rng = np.random.default_rng(seed)
    g = {"linear": Gradient.linear(11 * k, 7 * k, 230 * k, 83 * k, method=method),
         "radial": Gradient.radial(120 * k, 40 * k, 6 * k, 130 * k, 52 * k, 140 * k, method=method),
         "conic": Gradient.conic(128 * k, 48 * k, 0.9, method=method)}[kind]
    for off in sorted(rng.uniform(0, 1, n_stops)):
        c = rng.uniform(0, 1, 4)
        space = ("rgb", "srgb", "hsl")[int(rng.integers(0, 3))]
        col = Color.hsl(c[0] * 360, c[1], c[2], c[3]) if space == "hsl" else getattr(Color, space)(*map(float, c))
        g.add_stop(float(off), col)
    return g


@pytest.mark.parametrize("precision", ["integer", "float"])
@pytest.mark.parametrize("dither", ["none", "bayer", "blue_noise"])
@pytest.mark.parametrize("method", ["linear_rgb", "srgb", "hsl"])
@pytest.mark.parametrize("kind", ["linear", "radial", "conic"])
def test_mask_batch_gradient_source(gpu, oracle, kind, method, dither, precision):
    seed = zlib.crc32(f"{kind}/{method}/{dither}".encode()) % 1000
    g = _gradient(kind, method, 2 + seed % 7, seed)
    src = Pattern.from_gradient(g) if dither == "none" else Pattern.dither(dither, g, 8)
    for fmt, op in (("rgba", "src_over"), ("rgb", "multiply"), ("alpha8", "xor"), ("alpha2", "src_over")):
        ops = [Operation("dst_in", dst=src, src=_mask(W, H, seed)), Operation(op)]
        _check(gpu, oracle, fmt, ops, precision, seed=seed, what=f"{kind}/{method}/{dither}/{precision}/{fmt}/{op}")


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("op", ["src_over", "xor", "multiply", "hard_light", "color_dodge", "hue"])
def test_surface_source(gpu, oracle, fmt, op):
    """Surface.composite with a whole-surface source of another format."""
    src = _surface("rgba", W, H, 99)
    _check(gpu, oracle, fmt, [Operation(op, src=src)], "integer", seed=5, what=f"{fmt}/{op}")


@pytest.mark.parametrize("fmt,op,precision", [("rgba", "src_over", "integer"), ("rgba", "overlay", "float"),
                                              ("alpha8", "src_over", "integer"), ("alpha4", "dst_atop", "integer"),
                                              ("alpha1", "src_over", "integer"), ("alpha2", "xor", "integer")])
def test_mask_batch_1024(gpu, oracle, fmt, op, precision):
    n = 1024
    src = Pattern.from_pixel(Pixel.rgba(30, 200, 60, 230))
    ops = [Operation("dst_in", dst=src, src=_mask(n, n, 1)), Operation(op)]
    _check(gpu, oracle, fmt, ops, precision, w=n, h=n, seed=2, what=f"1024 {fmt}/{op}/{precision}")


def test_gradient_1024(gpu, oracle):
    n = 1024
    for kind, method in (("linear", "srgb"), ("conic", "linear_rgb"), ("radial", "hsl")):
        g = _gradient(kind, method, 8, 5, k=4.0)
        ops = [Operation("dst_in", dst=Pattern.dither("blue_noise", g, 8), src=_mask(n, n, 3)), Operation("src_over")]
        _check(gpu, oracle, "rgba", ops, "integer", w=n, h=n, seed=4, what=f"1024 {kind}/{method}")
