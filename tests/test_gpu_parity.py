"""Parity of the GPU path (through the C ABI) with the CPU oracle.

Every path must be bit-exact: integer pixels, float operators and
gradients alike (both sides compute in the same IEEE operation order, and
both restate the Zig standard library's pow and atan2 that z2d calls).
"""
import numpy as np
import pytest

from backends import GpuBackend
from scenes import FILL_SCENES, COMPOSITOR_SCENES
from z2d_gb300 import abi
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, FillOptions, Gradient, Operation, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background, random_fills, random_path, star_300

pytestmark = pytest.mark.gpu

FLOAT_TOL = 0  # float operators and gradients are bit-exact too (Zig's pow/atan2 restated on both sides)


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()


def _cmp(a: Surface, b: Surface, tol: int = 0, what: str = ""):
    x = a.numpy().astype(np.int16)
    y = b.numpy().astype(np.int16)
    assert x.shape == y.shape
    d = np.abs(x - y)
    ndiff = int((d > 0).sum())
    if tol == 0:
        assert ndiff == 0, f"{what}: {ndiff} bytes differ (max {int(d.max())})"
    else:
        assert int(d.max()) <= tol, f"{what}: max diff {int(d.max())} over {ndiff} bytes"
    return ndiff


@pytest.mark.parametrize("aa", ["none", "multisample_4x", "supersample_4x"])
@pytest.mark.parametrize("name", list(FILL_SCENES))
def test_fill_scene(gpu, oracle, name, aa):
    _cmp(FILL_SCENES[name](gpu, aa), FILL_SCENES[name](oracle, aa), 0, name)


@pytest.mark.parametrize("name", list(COMPOSITOR_SCENES))
def test_compositor_scene(gpu, oracle, name):
    _cmp(COMPOSITOR_SCENES[name](gpu), COMPOSITOR_SCENES[name](oracle), 0, name)


def test_star_300(gpu, oracle):
    w, h, nodes, pat, opts = star_300()
    a, b = Surface.init("rgba", w, h), Surface.init("rgba", w, h)
    assert gpu.fill(a, pat, nodes, opts) == abi.OK
    assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, "star")


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


FORMATS = ["rgba", "argb", "rgb", "xrgb", "alpha8", "alpha4", "alpha2", "alpha1"]


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("aa", ["none", "default"])
def test_random_fills_pixel_src_over(gpu, oracle, fmt, aa):
    w, h = 173, 131  # odd sizes: rows of packed formats are not byte aligned
    fills = random_fills(seed=7, n=12, w=w, h=h, side_lo=4, side_hi=160, seg_lo=3, seg_hi=24)
    a, b = _bg(fmt, w, h, 1), _bg(fmt, w, h, 1)
    for pat, nodes, opts in fills:
        opts.anti_aliasing = aa
        assert gpu.fill(a, pat, nodes, opts) == abi.OK
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, f"{fmt}/{aa}")


INT_OPS = [o for o in abi.OPERATORS if o not in abi.FLOAT_ONLY_OPS]


@pytest.mark.parametrize("op", abi.OPERATORS)
@pytest.mark.parametrize("aa", ["none", "default"])
def test_random_fills_all_operators(gpu, oracle, op, aa):
    w, h = 120, 90
    fills = random_fills(seed=abi.OP[op] + 100, n=4, w=w, h=h, side_lo=10, side_hi=100, seg_lo=3, seg_hi=12)
    a, b = _bg("rgba", w, h, 2), _bg("rgba", w, h, 2)
    for pat, nodes, opts in fills:
        opts.anti_aliasing = aa
        opts.operator = op
        assert gpu.fill(a, pat, nodes, opts) == abi.OK
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, FLOAT_TOL if op in abi.FLOAT_ONLY_OPS else 0, op)


def _gradients():
    lin = Gradient.linear(5, 7, 110, 80)
    rad = Gradient.radial(60, 45, 5, 55, 40, 70)
    con = Gradient.conic(60, 45, 0.7)
    hsl = Gradient.linear(0, 0, 120, 90, method="hsl", polar="longer")
    srgb = Gradient.radial(30, 30, 0, 60, 45, 80, method="srgb")
    for g in (lin, rad, con, hsl, srgb):
        g.add_stop(0.0, Color.rgb(1, 0, 0, 0.9))
        g.add_stop(0.35, Color.rgb(0, 1, 0.2, 0.5))
        g.add_stop(0.8, Color.hsl(200, 0.7, 0.4, 1.0))
        g.add_stop(1.0, Color.srgb(0.1, 0.2, 0.9, 0.75))
    return {"linear": lin, "radial": rad, "conic": con, "hsl": hsl, "srgb": srgb}


@pytest.mark.parametrize("gname", ["linear", "radial", "conic", "hsl", "srgb"])
@pytest.mark.parametrize("dither", ["none", "bayer", "blue_noise"])
@pytest.mark.parametrize("precision", ["integer", "float"])
def test_gradient_fills(gpu, oracle, gname, dither, precision):
    g = _gradients()[gname]
    pat = Pattern.from_gradient(g) if dither == "none" else Pattern.dither(dither, g, 8)
    w, h = 120, 90
    rng = np.random.default_rng(11)
    a, b = _bg("rgba", w, h, 3), _bg("rgba", w, h, 3)
    for i in range(3):
        nodes = random_path(rng, w, h, 20, 110, 3, 10)
        opts = FillOptions(precision=precision, operator="src_over" if i != 1 else "multiply")
        assert gpu.fill(a, pat, nodes, opts) == abi.OK
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    n = _cmp(a, b, FLOAT_TOL, f"{gname}/{dither}/{precision}")
    print(f"{gname}/{dither}/{precision}: {n} bytes differ by 1")


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("op", abi.OPERATORS)
def test_composite_mask_batch(gpu, oracle, fmt, op):
    """The compositor sweep kernel: [dst_in(dst=source, src=mask), op]."""
    w, h = 67, 29
    rng = np.random.default_rng(abi.OP[op])
    mask = Surface.init("alpha8", w, h)
    mask.data[:] = rng.integers(0, 256, size=mask.data.size, dtype=np.uint8)
    src = Pattern.from_pixel(Pixel.rgba(90, 40, 160, 200))
    ops = [Operation("dst_in", dst=src, src=mask), Operation(op)]
    a, b = _bg(fmt, w, h, 4), _bg(fmt, w, h, 4)
    assert gpu.composite(a, 0, 0, ops) == abi.OK
    assert oracle.composite(b, 0, 0, ops) == abi.OK
    _cmp(a, b, FLOAT_TOL if op in abi.FLOAT_ONLY_OPS else 0, f"{fmt}/{op}")


@pytest.mark.parametrize("offset", [(0, 0), (5, 3), (-7, -2), (40, 20)])
@pytest.mark.parametrize("fmt", ["rgba", "alpha4", "alpha1"])
def test_composite_surface_offsets(gpu, oracle, offset, fmt):
    w, h = 64, 48
    src = _bg("rgba", 37, 23, 5)
    a, b = _bg(fmt, w, h, 6), _bg(fmt, w, h, 6)
    ops = [Operation("src_over", src=src)]
    assert gpu.composite(a, offset[0], offset[1], ops) == abi.OK
    assert oracle.composite(b, offset[0], offset[1], ops) == abi.OK
    _cmp(a, b, 0, f"{fmt}/{offset}")


def test_fill_batch_matches_sequential(oracle):
    from z2d_gb300 import painter
    w, h = 512, 384
    fills = random_fills(seed=3, n=150, w=w, h=h, side_lo=8, side_hi=300, seg_lo=3, seg_hi=40)
    a, b = _bg("rgba", w, h, 8), _bg("rgba", w, h, 8)
    painter.fill_batch(a, fills)
    for pat, nodes, opts in fills:
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, "batch")


def test_device_surface(oracle):
    torch = pytest.importorskip("torch")
    from z2d_gb300 import painter
    w, h, nodes, pat, opts = star_300()
    a = Surface.init("rgba", w, h).to_device("cuda")
    painter.fill(a, pat, nodes, opts)
    torch.cuda.synchronize()
    b = Surface.init("rgba", w, h)
    oracle.fill(b, pat, nodes, opts)
    _cmp(a.to_host(), b, 0, "device star")


def test_errors(gpu):
    s = Surface.init("rgba", 10, 10)
    open_path = [(abi.MOVE_TO, 1, 1, 0, 0, 0, 0), (abi.LINE_TO, 5, 5, 0, 0, 0, 0)]
    assert gpu.fill(s, Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4)), open_path, FillOptions()) == abi.ERR_PATH_NOT_CLOSED
    closed = open_path + [(abi.LINE_TO, 1, 5, 0, 0, 0, 0), (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)]
    bad_px = Pattern.from_pixel(Pixel.rgba(200, 2, 3, 4))
    assert gpu.fill(s, bad_px, closed, FillOptions()) == abi.ERR_PIXEL_NOT_PREMULTIPLIED
    no_move = [(abi.LINE_TO, 5, 5, 0, 0, 0, 0), (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)]
    assert gpu.fill(s, Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4)), no_move, FillOptions()) == abi.ERR_INVALID_STATE
    assert gpu.fill(s, Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4)), [], FillOptions()) == abi.OK


@pytest.mark.parametrize("n_stops", [33, 100, 257])
@pytest.mark.parametrize("method", ["linear_rgb", "srgb", "hsl"])
def test_gradient_many_stops(gpu, oracle, n_stops, method):
    """z2d's stop list has no length limit (src/gradient.zig:183-198): stop
    lists beyond the 32 held inline travel as tables beside the
    descriptors, through fills, the compositor and a dither source."""
    rng = np.random.default_rng(n_stops)
    g = Gradient.linear(3, 9, 150, 70, method=method)
    for off in rng.uniform(-0.1, 1.1, n_stops):  # unsorted, some clamped, some repeated
        c = rng.uniform(0, 1, 4)
        g.add_stop(float(round(off, 2)), Color.rgb(*map(float, c)))
    w, h = 160, 80
    a, b = _bg("rgba", w, h, 12), _bg("rgba", w, h, 12)
    for i, pat in enumerate((Pattern.from_gradient(g), Pattern.dither("bayer", g, 8))):
        nodes = random_path(rng, w, h, 30, 150, 3, 12)
        opts = FillOptions(precision="float" if i else "integer")
        assert gpu.fill(a, pat, nodes, opts) == abi.OK
        assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, f"fill {n_stops}")
    ops = [Operation("src_over", src=Pattern.from_gradient(g))]
    assert gpu.composite(a, 0, 0, ops) == abi.OK
    assert oracle.composite(b, 0, 0, ops) == abi.OK
    _cmp(a, b, 0, f"composite {n_stops}")


@pytest.mark.parametrize("rule", ["non_zero", "even_odd"])
@pytest.mark.parametrize("aa", ["none", "default", "supersample_4x"])
def test_unbalanced_rows_many_active_edges(gpu, oracle, rule, aa):
    """Closed two-point subpaths add one edge each and leave rows unbalanced,
    which z2d draws with its literal sorted-span loop (the GPU's exact path).
    Here 33 such edges cross the same rows, in pairs at equal x with opposite
    directions, so more than 24 crossings of a row are sorted and ties must
    be ordered.  z2d sorts them with std.sort.pdqContext, which is not in the
    reference tree; the oracle and the GPU both order ties stably, and this
    pins that they agree on every pixel."""
    w, h = 200, 100
    nodes = []
    for k in range(33):
        x = 4.0 + 5.5 * (k // 2)
        y0, y1 = (8.0, 92.0) if k % 2 == 0 else (93.0, 7.0)  # opposite directions at the same x
        nodes += [(abi.MOVE_TO, x, y0, 0, 0, 0, 0), (abi.LINE_TO, x + 0.25 * (k % 3), y1, 0, 0, 0, 0),
                  (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)]
    nodes += [(abi.MOVE_TO, 1.0, 50.0, 0, 0, 0, 0), (abi.LINE_TO, 199.0, 50.5, 0, 0, 0, 0), (abi.LINE_TO, 100.0, 99.0, 0, 0, 0, 0),
              (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)]
    pat = Pattern.from_pixel(Pixel.rgba(40, 90, 140, 230))
    opts = FillOptions(anti_aliasing=aa, fill_rule=rule)
    a, b = _bg("rgba", w, h, 13), _bg("rgba", w, h, 13)
    assert gpu.fill(a, pat, nodes, opts) == abi.OK
    assert oracle.fill(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, f"{rule}/{aa}")
