"""painter.stroke on the GPU (z2dgpu_stroke) against the oracle rasterising
the same stroke polygon (StrokeOracle).  The polygon builder itself is
pinned to z2d by the stroke scenes' golden PNGs (test_oracle_golden.py)."""
import math

import numpy as np
import pytest

from backends import GpuBackend, StrokeOracle
from scenes import STROKE_SCENES
from z2d_gb300 import abi
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, Gradient, Pattern, Pixel, StrokeOptions
from z2d_gb300.workloads import premultiplied_background, random_path, random_premultiplied_pixel

pytestmark = pytest.mark.gpu

FLOAT_TOL = 0  # float operators and gradients: bit-exact


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()


def _cmp(a, b, tol, what):
    d = np.abs(a.numpy().astype(np.int16) - b.numpy().astype(np.int16))
    assert int(d.max(initial=0)) <= tol, f"{what}: {int((d > 0).sum())} bytes differ (max {int(d.max())})"


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


@pytest.mark.parametrize("aa", ["none", "multisample_4x", "supersample_4x"])
@pytest.mark.parametrize("name", list(STROKE_SCENES))
def test_stroke_scene(gpu, oracle, name, aa):
    _cmp(STROKE_SCENES[name](gpu, aa), STROKE_SCENES[name](StrokeOracle(oracle), aa), 0, name)


def _open_path(rng, w, h, n):
    pts = [(abi.MOVE_TO, *rng.uniform([5, 5], [w - 5, h - 5]), 0, 0, 0, 0)]
    for _ in range(n):
        if rng.random() < 0.6:
            pts.append((abi.LINE_TO, *rng.uniform([5, 5], [w - 5, h - 5]), 0, 0, 0, 0))
        else:
            pts.append((abi.CURVE_TO, *rng.uniform([5, 5, 5, 5, 5, 5], [w - 5, h - 5] * 3)))
    return pts


TRANSFORMS = {
    "identity": (1, 0, 0, 1, 0, 0),
    "scale": (1.5, 0, 0, 0.75, 3, -2),
    "rotate": (math.cos(0.4), -math.sin(0.4), math.sin(0.4), math.cos(0.4), 0, 0),
    "skew_flip": (1.0, 0.3, 0.2, -1.1, 0, 0),
}


@pytest.mark.parametrize("tf", list(TRANSFORMS))
@pytest.mark.parametrize("join", ["miter", "round", "bevel"])
@pytest.mark.parametrize("cap", ["butt", "round", "square"])
def test_random_strokes(gpu, oracle, join, cap, tf):
    rng = np.random.default_rng(hash((join, cap, tf)) & 0xFFFF)
    w, h = 160, 120
    a, b = _bg("rgba", w, h, 3), _bg("rgba", w, h, 3)
    so = StrokeOracle(oracle)
    for i in range(4):
        nodes = _open_path(rng, w, h, int(rng.integers(1, 6)))
        if i % 2:
            nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
        opts = StrokeOptions(line_join=join, line_cap=cap, line_width=float(rng.choice([0.5, 1.5, 3.0, 7.0, 12.0])),
                             miter_limit=float(rng.choice([1.0, 4.0, 10.0])), transformation=TRANSFORMS[tf],
                             anti_aliasing=("default", "none", "supersample_4x")[i % 3])
        pat = Pattern.from_pixel(random_premultiplied_pixel(rng))
        assert gpu.stroke(a, pat, nodes, opts) == abi.OK
        assert so.stroke(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, f"{join}/{cap}/{tf}")


@pytest.mark.parametrize("fmt", ["rgb", "alpha8", "alpha4", "alpha1"])
@pytest.mark.parametrize("op", ["src_over", "src_in", "xor", "color_burn"])
def test_stroke_formats_operators(gpu, oracle, fmt, op):
    rng = np.random.default_rng(abi.OP[op] * 10 + len(fmt))
    w, h = 97, 71
    a, b = _bg(fmt, w, h, 5), _bg(fmt, w, h, 5)
    g = Gradient.linear(0, 0, w, h)
    g.add_stop(0.0, Color.rgb(1, 0.2, 0, 0.9))
    g.add_stop(1.0, Color.rgb(0, 0.3, 1, 0.6))
    so = StrokeOracle(oracle)
    for i in range(3):
        nodes = _open_path(rng, w, h, 3)
        opts = StrokeOptions(line_join="round", line_cap="square", line_width=5.0, operator=op,
                             precision="float" if i == 2 else "integer")
        pat = Pattern.from_gradient(g) if i == 1 else Pattern.from_pixel(random_premultiplied_pixel(rng))
        assert gpu.stroke(a, pat, nodes, opts) == abi.OK
        assert so.stroke(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, FLOAT_TOL, f"{fmt}/{op}")


def test_stroke_degenerate_paths(gpu, oracle):
    so = StrokeOracle(oracle)
    cases = [
        [(abi.MOVE_TO, 20, 20, 0, 0, 0, 0), (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)],                     # dot
        [(abi.MOVE_TO, 20, 20, 0, 0, 0, 0), (abi.LINE_TO, 20, 20, 0, 0, 0, 0)],                      # zero length
        [(abi.MOVE_TO, 10, 10, 0, 0, 0, 0), (abi.LINE_TO, 50, 10, 0, 0, 0, 0),
         (abi.LINE_TO, 90, 10, 0, 0, 0, 0)],                                                           # colinear
        [(abi.MOVE_TO, 10, 40, 0, 0, 0, 0), (abi.LINE_TO, 60, 40, 0, 0, 0, 0),
         (abi.LINE_TO, 10, 40, 0, 0, 0, 0)],                                                           # reversal
        [(abi.MOVE_TO, 30, 30, 0, 0, 0, 0), (abi.LINE_TO, 70, 60, 0, 0, 0, 0),
         (abi.LINE_TO, 30, 30, 0, 0, 0, 0), (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)],                     # closed back
    ]
    for cap in ("butt", "round", "square"):
        for k, nodes in enumerate(cases):
            a, b = _bg("rgba", 100, 80, k), _bg("rgba", 100, 80, k)
            opts = StrokeOptions(line_cap=cap, line_join="round", line_width=9.0)
            pat = Pattern.from_pixel(Pixel.rgba(200, 100, 50, 255))
            assert gpu.stroke(a, pat, nodes, opts) == abi.OK
            assert so.stroke(b, pat, nodes, opts) == abi.OK
            _cmp(a, b, 0, f"case {k} {cap}")


def _multi_subpath_path(rng, w, h):
    """Several subpaths of every kind the plotter distinguishes: open and
    closed polylines with curves, lone points, dots, curves whose control
    points coincide with their ends, paths that return to their start."""
    nodes = []
    for _ in range(int(rng.integers(2, 6))):
        kind = rng.integers(0, 6)
        x, y = rng.uniform([8, 8], [w - 8, h - 8])
        nodes.append((abi.MOVE_TO, x, y, 0, 0, 0, 0))
        if kind == 0:  # lone move_to or dot
            if rng.random() < 0.5:
                nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
            continue
        for _ in range(int(rng.integers(1, 7))):
            r = rng.random()
            if r < 0.45:
                nodes.append((abi.LINE_TO, *rng.uniform([8, 8], [w - 8, h - 8]), 0, 0, 0, 0))
            elif r < 0.55:  # repeated point
                last = nodes[-1][1:3] if nodes[-1][0] != abi.CURVE_TO else nodes[-1][5:7]
                nodes.append((abi.LINE_TO, *last, 0, 0, 0, 0))
            elif r < 0.65:  # degenerate control points
                last = nodes[-1][1:3] if nodes[-1][0] != abi.CURVE_TO else nodes[-1][5:7]
                e = rng.uniform([8, 8], [w - 8, h - 8])
                nodes.append((abi.CURVE_TO, *last, *e, *e))
            else:
                nodes.append((abi.CURVE_TO, *rng.uniform([8, 8, 8, 8, 8, 8], [w - 8, h - 8] * 3)))
        if kind == 5:
            nodes.append((abi.LINE_TO, x, y, 0, 0, 0, 0))  # back to the start
        if kind >= 3:
            nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
    return nodes


@pytest.mark.parametrize("seed", range(6))
def test_multi_subpath_strokes(gpu, oracle, seed):
    rng = np.random.default_rng(900 + seed)
    w, h = 180, 140
    a, b = _bg("rgba", w, h, seed), _bg("rgba", w, h, seed)
    so = StrokeOracle(oracle)
    tfs = list(TRANSFORMS.values())
    for i in range(6):
        nodes = _multi_subpath_path(rng, w, h)
        opts = StrokeOptions(line_join=("miter", "round", "bevel")[i % 3], line_cap=("butt", "round", "square")[i // 2 % 3],
                             line_width=float(rng.choice([0.3, 1.0, 2.0, 4.5, 9.0, 16.0])),
                             miter_limit=float(rng.choice([1.2, 4.0, 10.0])), transformation=tfs[i % len(tfs)],
                             tolerance=float(rng.choice([0.05, 0.1, 0.5])))
        pat = Pattern.from_pixel(random_premultiplied_pixel(rng))
        assert gpu.stroke(a, pat, nodes, opts) == abi.OK
        assert so.stroke(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, f"seed {seed}")


def test_stroke_node_sequence_errors(gpu):
    s = Surface.init("rgba", 20, 20)
    px = Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4))
    m, l, c, z = abi.MOVE_TO, abi.LINE_TO, abi.CURVE_TO, abi.CLOSE_PATH
    bad = [
        [(l, 1, 1, 0, 0, 0, 0), (l, 5, 5, 0, 0, 0, 0)],                                   # no current point
        [(m, 1, 1, 0, 0, 0, 0), (l, 5, 5, 0, 0, 0, 0), (z, 0, 0, 0, 0, 0, 0), (l, 9, 9, 0, 0, 0, 0)],
        [(m, 1, 1, 0, 0, 0, 0), (z, 0, 0, 0, 0, 0, 0), (c, 1, 2, 3, 4, 5, 6)],
        [(m, 1, 1, 0, 0, 0, 0), (l, float("nan"), 5, 0, 0, 0, 0)],
    ]
    for nodes in bad:
        assert gpu.stroke(s, px, nodes, StrokeOptions(line_width=3.0)) == abi.ERR_INVALID_STATE, nodes
    ok = [(z, 0, 0, 0, 0, 0, 0), (m, 3, 3, 0, 0, 0, 0), (z, 0, 0, 0, 0, 0, 0), (z, 0, 0, 0, 0, 0, 0), (m, 4, 4, 0, 0, 0, 0)]
    assert gpu.stroke(s, px, ok, StrokeOptions(line_width=3.0)) == abi.OK


def test_stroke_errors(gpu):
    s = Surface.init("rgba", 10, 10)
    nodes = [(abi.MOVE_TO, 1, 1, 0, 0, 0, 0), (abi.LINE_TO, 8, 8, 0, 0, 0, 0)]
    px = Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4))
    assert gpu.stroke(s, px, nodes, StrokeOptions(transformation=(1, 2, 2, 4, 0, 0))) == abi.ERR_INVALID_ARGUMENT
    assert gpu.stroke(s, Pattern.from_pixel(Pixel.rgba(200, 2, 3, 4)), nodes,
                      StrokeOptions()) == abi.ERR_PIXEL_NOT_PREMULTIPLIED
    assert gpu.stroke(s, px, nodes, StrokeOptions(hairline=True)) == abi.OK
    assert gpu.stroke(s, px, [], StrokeOptions()) == abi.OK
    assert gpu.stroke(s, px, nodes, StrokeOptions(dashes=(0.0, 0.0))) == abi.OK  # invalid dashes: solid stroke


@pytest.mark.parametrize("dashes,offset", [((10.0, 5.0), 0.0), ((3.0, 1.0, 0.0, 2.0), 1.5), ((7.0,), -2.0),
                                           ((0.0, 4.0), 0.0), ((2.5, 2.5), 40.0)])
@pytest.mark.parametrize("cap", ["butt", "round", "square"])
def test_dashed_strokes(gpu, oracle, dashes, offset, cap):
    rng = np.random.default_rng(int(sum(dashes) * 10 + offset * 3) + len(cap))
    w, h = 150, 110
    a, b = _bg("rgba", w, h, 7), _bg("rgba", w, h, 7)
    so = StrokeOracle(oracle)
    for i in range(4):
        nodes = _open_path(rng, w, h, int(rng.integers(1, 6)))
        if i % 2:
            nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
        opts = StrokeOptions(line_cap=cap, line_join=("miter", "round", "bevel")[i % 3], line_width=4.0 + i,
                             dashes=dashes, dash_offset=offset,
                             transformation=TRANSFORMS[("identity", "scale", "rotate", "skew_flip")[i]])
        pat = Pattern.from_pixel(random_premultiplied_pixel(rng))
        assert gpu.stroke(a, pat, nodes, opts) == abi.OK
        assert so.stroke(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, 0, f"{dashes}/{offset}/{cap}")


def _dash_path(rng, w, h):
    """Subpaths of lines and curves, some closed, with repeated points and
    points returning to the start (the dasher's degenerate cases)."""
    nodes = []
    for _ in range(int(rng.integers(1, 4))):
        start = rng.uniform([5, 5], [w - 5, h - 5])
        nodes.append((abi.MOVE_TO, *start, 0, 0, 0, 0))
        last = start
        for _ in range(int(rng.integers(1, 7))):
            r = rng.random()
            if r < 0.1:  # the same point again
                nodes.append((abi.LINE_TO, *last, 0, 0, 0, 0))
            elif r < 0.55:
                last = rng.uniform([5, 5], [w - 5, h - 5])
                nodes.append((abi.LINE_TO, *last, 0, 0, 0, 0))
            else:
                c = rng.uniform([5, 5, 5, 5, 5, 5], [w - 5, h - 5] * 3)
                nodes.append((abi.CURVE_TO, *c))
                last = c[4:]
        if rng.random() < 0.2:
            nodes.append((abi.LINE_TO, *start, 0, 0, 0, 0))
        if rng.random() < 0.5:
            nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
    return nodes


@pytest.mark.parametrize("seed", range(4))
def test_dashed_random_batch(oracle, seed):
    """Dashed strokes with random dash arrays (zero-length entries
    included), offsets, caps, joins, widths and transforms, drawn in one
    z2dgpu_draw_jobs call over many surfaces (their polygons uploaded and
    rasterised with the fills), against the oracle's rasteriser."""
    torch = pytest.importorskip("torch")
    from z2d_gb300 import painter
    so = StrokeOracle(oracle)
    rng = np.random.default_rng(4242 + seed)
    jobs, refs = [], []
    for j in range(24):
        w, h = int(rng.integers(40, 160)), int(rng.integers(40, 120))
        dev = _bg("rgba", w, h, 700 + j).to_device("cuda")
        ref = _bg("rgba", w, h, 700 + j)
        ops = []
        for k in range(5):
            nd = int(rng.integers(1, 6))
            dashes = tuple(float(v) if rng.random() > 0.2 else 0.0 for v in rng.uniform(0.5, 25.0, nd))
            if not any(dashes):
                dashes = (4.0,) + dashes[1:]
            offset = float(rng.choice([0.0, rng.uniform(-30, 30), rng.uniform(0, 200)]))
            opts = StrokeOptions(line_width=float(rng.uniform(0.5, 14)),
                                 line_join=("miter", "round", "bevel")[int(rng.integers(0, 3))],
                                 line_cap=("butt", "round", "square")[int(rng.integers(0, 3))],
                                 miter_limit=float(rng.uniform(1.0, 12.0)),
                                 dashes=dashes, dash_offset=offset,
                                 transformation=TRANSFORMS[list(TRANSFORMS)[int(rng.integers(0, 4))]])
            ops.append(("stroke", Pattern.from_pixel(random_premultiplied_pixel(rng)), _dash_path(rng, w, h), opts))
        for kind, pat, nodes, o in ops:
            assert so.stroke(ref, pat, nodes, o) == abi.OK
        jobs.append((dev, ops))
        refs.append(ref)
    painter.draw_jobs(jobs)
    torch.cuda.synchronize()
    for j, ((dev, _), ref) in enumerate(zip(jobs, refs)):
        _cmp(dev.to_host(), ref, 0, f"job {j}")


def test_draw_jobs_mixed(oracle):
    """z2dgpu_draw_jobs: fills and strokes (dashed or not) interleaved over
    many surfaces equal the same calls one by one."""
    torch = pytest.importorskip("torch")
    from z2d_gb300 import painter
    from z2d_gb300.types import FillOptions
    from z2d_gb300.workloads import random_fills
    so = StrokeOracle(oracle)
    rng = np.random.default_rng(99)
    jobs, refs = [], []
    for j in range(20):
        w, h = int(rng.integers(20, 180)), int(rng.integers(20, 140))
        fmt = ("rgba", "rgb", "alpha8", "alpha4")[j % 4]
        dev = _bg(fmt, w, h, 500 + j).to_device("cuda")
        ref = _bg(fmt, w, h, 500 + j)
        ops = []
        fills = random_fills(seed=900 + j, n=int(rng.integers(0, 6)), w=w, h=h, side_lo=2, side_hi=max(3, min(w, h)),
                             seg_lo=3, seg_hi=10)
        for k, (pat, nodes, fo) in enumerate(fills):
            ops.append(("fill", pat, nodes, fo))
            if k % 2 == 0:
                sn = _open_path(rng, w, h, int(rng.integers(1, 5)))
                st = StrokeOptions(line_width=float(rng.uniform(0.5, 12)), line_join=("miter", "round", "bevel")[k % 3],
                                   line_cap=("butt", "round", "square")[(k + j) % 3],
                                   dashes=(6.0, 3.0) if (k + j) % 4 == 0 else (),
                                   anti_aliasing=("default", "none", "supersample_4x")[j % 3])
                ops.append(("stroke", Pattern.from_pixel(random_premultiplied_pixel(rng)), sn, st))
        for kind, pat, nodes, o in ops:
            rc = oracle.fill(ref, pat, nodes, o) if kind == "fill" else so.stroke(ref, pat, nodes, o)
            assert rc == abi.OK
        jobs.append((dev, ops))
        refs.append(ref)
    painter.draw_jobs(jobs)
    torch.cuda.synchronize()
    for j, ((dev, _), ref) in enumerate(zip(jobs, refs)):
        _cmp(dev.to_host(), ref, 0, f"job {j}")


def _hairline_path(rng, w, h):
    """Polylines that cross themselves and leave the surface: lines, curves,
    lone points, closed and open subpaths."""
    nodes = []
    for _ in range(int(rng.integers(1, 4))):
        nodes.append((abi.MOVE_TO, *rng.uniform([-20, -20], [w + 20, h + 20]), 0, 0, 0, 0))
        if rng.random() < 0.15:  # a lone point
            nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
            continue
        for _ in range(int(rng.integers(1, 7))):
            if rng.random() < 0.7:
                nodes.append((abi.LINE_TO, *rng.uniform([-20, -20], [w + 20, h + 20]), 0, 0, 0, 0))
            else:
                nodes.append((abi.CURVE_TO, *rng.uniform([-20, -20] * 3, [w + 20, h + 20] * 3)))
        if rng.random() < 0.5:
            nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
    return nodes


@pytest.mark.parametrize("aa", ["none", "default"])
@pytest.mark.parametrize("fmt", ["rgba", "rgb", "alpha8", "alpha4", "alpha1"])
def test_hairlines(gpu, oracle, fmt, aa):
    """Hairline strokes (Bresenham / Wu segments composited pixel by pixel
    in path order) against the oracle's hairline rasteriser."""
    rng = np.random.default_rng(len(fmt) * 7 + (aa == "none"))
    w, h = 120, 90
    a, b = _bg(fmt, w, h, 21), _bg(fmt, w, h, 21)
    so = StrokeOracle(oracle)
    g = Gradient.linear(0, 0, w, h)
    g.add_stop(0.0, Color.rgb(1, 0.2, 0, 0.9))
    g.add_stop(1.0, Color.rgb(0, 0.3, 1, 0.6))
    for i in range(8):
        nodes = _hairline_path(rng, w, h)
        op = ("src_over", "src", "xor", "plus", "src_in", "clear", "color_burn", "multiply")[i]
        opts = StrokeOptions(hairline=True, anti_aliasing=aa, operator=op,
                             dashes=(7.0, 3.0) if i % 3 == 2 else (), dash_offset=1.5,
                             precision="float" if i == 7 else "integer", tolerance=(0.1, 0.5)[i % 2])
        pat = Pattern.from_gradient(g) if i % 4 == 1 else Pattern.from_pixel(random_premultiplied_pixel(rng))
        assert gpu.stroke(a, pat, nodes, opts) == abi.OK
        assert so.stroke(b, pat, nodes, opts) == abi.OK
    _cmp(a, b, FLOAT_TOL, f"{fmt}/{aa}")


def test_hairline_star_overdraw(gpu, oracle):
    """Segments crossing many times at one pixel with a translucent source:
    the composites must apply in path order."""
    s_gpu, s_ref = _bg("rgba", 64, 64, 3), _bg("rgba", 64, 64, 3)
    nodes = [(abi.MOVE_TO, 32, 2, 0, 0, 0, 0)]
    for k in range(1, 40):
        t = k * 2.513
        nodes.append((abi.LINE_TO, 32 + 30 * math.sin(t), 32 - 30 * math.cos(t), 0, 0, 0, 0))
    nodes.append((abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0))
    pat = Pattern.from_pixel(Pixel.rgba(40, 20, 10, 90))
    so = StrokeOracle(oracle)
    for aa in ("none", "default"):
        opts = StrokeOptions(hairline=True, anti_aliasing=aa, operator="src_over")
        assert gpu.stroke(s_gpu, pat, nodes, opts) == abi.OK
        assert so.stroke(s_ref, pat, nodes, opts) == abi.OK
    _cmp(s_gpu, s_ref, 0, "star")


def test_draw_jobs_with_hairlines(oracle):
    """Hairlines interleaved with fills and strokes on many surfaces keep
    each surface's call order."""
    torch = pytest.importorskip("torch")
    from z2d_gb300 import painter
    from z2d_gb300.workloads import random_fills
    so = StrokeOracle(oracle)
    rng = np.random.default_rng(321)
    jobs, refs = [], []
    for j in range(12):
        w, h = int(rng.integers(20, 150)), int(rng.integers(20, 120))
        fmt = ("rgba", "rgb", "alpha8")[j % 3]
        dev = _bg(fmt, w, h, 700 + j).to_device("cuda")
        ref = _bg(fmt, w, h, 700 + j)
        ops = []
        fills = random_fills(seed=1300 + j, n=int(rng.integers(1, 5)), w=w, h=h, side_lo=2,
                             side_hi=max(3, min(w, h)), seg_lo=3, seg_hi=8)
        for k, (pat, nodes, fo) in enumerate(fills):
            ops.append(("fill", pat, nodes, fo))
            if (k + j) % 2 == 0:
                ops.append(("stroke", Pattern.from_pixel(random_premultiplied_pixel(rng)), _hairline_path(rng, w, h),
                            StrokeOptions(hairline=True, anti_aliasing=("none", "default")[k % 2])))
            if k % 3 == 1:
                ops.append(("stroke", Pattern.from_pixel(random_premultiplied_pixel(rng)),
                            _open_path(rng, w, h, 3), StrokeOptions(line_width=3.0)))
        if j % 4 == 0:  # consecutive hairlines at the end
            for _ in range(2):
                ops.append(("stroke", Pattern.from_pixel(random_premultiplied_pixel(rng)), _hairline_path(rng, w, h),
                            StrokeOptions(hairline=True)))
        for kind, pat, nodes, o in ops:
            rc = oracle.fill(ref, pat, nodes, o) if kind == "fill" else so.stroke(ref, pat, nodes, o)
            assert rc == abi.OK
        jobs.append((dev, ops))
        refs.append(ref)
    painter.draw_jobs(jobs)
    torch.cuda.synchronize()
    for j, ((dev, _), ref) in enumerate(zip(jobs, refs)):
        _cmp(dev.to_host(), ref, 0, f"job {j}")
