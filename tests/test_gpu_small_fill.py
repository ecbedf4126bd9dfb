"""The one-upload path for few short fills against the pipeline and the oracle.

A call whose fills are few and short flattens and bins on the host and
launches only the rasteriser (run_small_jobs); a call beyond its limits
takes the full device pipeline.  Each case draws the fill both ways (the
pipeline's batch adds a second fill of 4,200 nodes that lies off the
surface and draws nothing) and compares both surfaces with the oracle's,
byte for byte: lines and curves,
even-odd and non-zero, every operator class (bounded, unbounded, float
only), gradient sources, paths partly or wholly off the surface, negative
coordinates, horizontal and degenerate edges, repeated points, open
two-point chains (which the small path hands back to the pipeline), and
paths beyond its limits.
"""
import numpy as np
import pytest

from backends import GpuBackend
from z2d_gb300 import abi, painter
from z2d_gb300.path import Path
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, FillOptions, Gradient, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background, random_path

pytestmark = pytest.mark.gpu

W, H = 300, 200


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()


def _bg(seed, fmt="rgba"):
    s = Surface.init(fmt, W, H)
    if fmt in ("rgba", "argb"):
        s.data[:] = premultiplied_background(np.random.default_rng(seed), W, H)
    return s


def _off_surface():
    """Off the surface, and more nodes than the one-upload path takes."""
    p = Path()
    p.move_to(-5000, -5000)
    for k in range(4200):
        p.line_to(-4000 - (k % 7), -5000 + k * 0.01)
    p.close()
    return p.to_array()


def _check(gpu, oracle, pat, nodes, opts, seed=0, fmt="rgba", what="", small=None):
    """Draws the fill alone and in the pipeline's batch; `small` says whether
    the single call must take the one-upload path (at most one launch) or
    must not (None: either)."""
    a, b, c = _bg(seed, fmt), _bg(seed, fmt), _bg(seed, fmt)
    n0 = gpu.ctx.launch_count
    assert gpu.fill(a, pat, nodes, opts) == abi.OK
    n1 = gpu.ctx.launch_count
    painter.fill_batch(b, [(pat, nodes, opts), (pat, _off_surface(), opts)], ctx=gpu.ctx)
    n2 = gpu.ctx.launch_count
    assert oracle.fill(c, pat, nodes, opts) == abi.OK
    ca = c.numpy()
    assert np.array_equal(a.numpy(), ca), f"{what}: single call differs from the oracle"
    assert np.array_equal(b.numpy(), ca), f"{what}: pipeline differs from the oracle"
    assert n2 - n1 > 1, f"{what}: the batch did not take the pipeline"
    if small is not None:
        assert (n1 - n0 <= 1) == small, f"{what}: {n1 - n0} launches for the single call"


@pytest.mark.parametrize("seed", range(16))
def test_random_paths(gpu, oracle, seed):
    rng = np.random.default_rng(900 + seed)
    for k in range(6):
        nodes = random_path(rng, W, H, side_lo=4.0, side_hi=400.0)
        pat = Pattern.from_pixel(Pixel.rgba(200, 60, 30, 230))
        opts = FillOptions(fill_rule="even_odd" if k & 1 else "non_zero",
                           tolerance=float(rng.choice([0.1, 0.5, 0.01])))
        _check(gpu, oracle, pat, nodes, opts, seed=seed, what=f"{seed}/{k}")


@pytest.mark.parametrize("op", ["src_over", "src", "clear", "dst_in", "src_in", "dst_atop", "xor", "multiply",
                                "hard_light", "hue", "color_dodge"])
def test_operators(gpu, oracle, op):
    rng = np.random.default_rng(abi.OP[op])
    nodes = random_path(rng, W, H, side_lo=60.0, side_hi=250.0)
    for prec in ("integer", "float"):
        _check(gpu, oracle, Pattern.from_pixel(Pixel.rgba(30, 90, 160, 200)), nodes,
               FillOptions(operator=op, precision=prec), seed=3, what=f"{op}/{prec}")


@pytest.mark.parametrize("kind", ["linear", "radial", "conic"])
def test_gradient_source(gpu, oracle, kind):
    g = {"linear": Gradient.linear(10, 20, 280, 150), "radial": Gradient.radial(150, 100, 10, 160, 90, 140),
         "conic": Gradient.conic(150, 100, 0.7)}[kind]
    g.add_stop(0.0, Color.rgb(1, 0, 0, 1)).add_stop(0.5, Color.srgb(0, 1, 0, 0.5)).add_stop(1.0, Color.rgb(0, 0, 1, 1))
    nodes = random_path(np.random.default_rng(7), W, H, side_lo=150.0, side_hi=290.0)
    _check(gpu, oracle, Pattern.from_gradient(g), nodes, FillOptions(), what=kind)


def _poly(points, close=True):
    p = Path()
    p.move_to(*points[0])
    for q in points[1:]:
        p.line_to(*q)
    if close:
        p.close()
    return p.to_array()


@pytest.mark.parametrize("name,points", [
    ("partly off", [(-50, -30), (120, 40), (60, 260)]),
    ("wholly off", [(400, 10), (500, 10), (450, 90)]),
    ("negative", [(-10.5, -7.25), (30.75, -2.0), (5.0, 20.5)]),
    ("horizontal edges", [(10, 10), (200, 10), (200, 150), (10, 150)]),
    ("repeated points", [(20, 20), (20, 20), (180, 40), (180, 40), (90, 170), (90, 170)]),
    ("thin", [(10, 100), (290, 100.2), (10, 100.4)]),
    ("sub-pixel", [(50.1, 50.1), (50.6, 50.2), (50.3, 50.9)]),
    ("bottom-right edge", [(250, 150), (300, 150), (300, 200), (250, 200)]),
    ("open chain", [(10, 10), (200, 150)]),
])
def test_shapes(gpu, oracle, name, points):
    _check(gpu, oracle, Pattern.from_pixel(Pixel.rgba(0, 120, 240, 255)), _poly(points), FillOptions(), what=name,
           small=name != "open chain")


def test_curves_and_subpaths(gpu, oracle):
    p = Path()
    p.move_to(20, 180).curve_to(20, 20, 280, 20, 280, 180).close()
    p.move_to(100, 150).curve_to(100, 60, 200, 60, 200, 150).curve_to(200, 200, 100, 200, 100, 150).close()
    p.move_to(140, 100).curve_to(140, 100, 150, 110, 150, 110).line_to(160, 90).close()  # degenerate curve
    for rule in ("non_zero", "even_odd"):
        _check(gpu, oracle, Pattern.from_pixel(Pixel.rgba(90, 30, 120, 200)), p.to_array(),
               FillOptions(fill_rule=rule), what=rule, small=True)


def test_beyond_limits(gpu, oracle):
    """More nodes or edges than the one-upload path takes: the pipeline."""
    rng = np.random.default_rng(5)
    p = Path()
    p.move_to(150, 100)
    for _ in range(5000):
        p.line_to(*map(float, rng.uniform(0, [W, H])))
    p.close()
    _check(gpu, oracle, Pattern.from_pixel(Pixel.rgba(10, 200, 90, 255)), p.to_array(),
           FillOptions(fill_rule="even_odd"), what="5000 lines", small=False)
    q = Path()
    q.move_to(0, 0).curve_to(1e5, 0, -1e5, 200, 300, 200).close()  # many subdivision leaves
    _check(gpu, oracle, Pattern.from_pixel(Pixel.rgba(10, 200, 90, 255)), q.to_array(),
           FillOptions(tolerance=0.001), what="long curve", small=False)


@pytest.mark.parametrize("fmt", ["rgb", "alpha8", "xrgb", "argb"])
def test_formats(gpu, oracle, fmt):
    nodes = random_path(np.random.default_rng(11), W, H, side_lo=100.0, side_hi=280.0)
    _check(gpu, oracle, Pattern.from_pixel(Pixel.rgba(80, 80, 200, 220)), nodes, FillOptions(), fmt=fmt, what=fmt)


def _dev_jobs(oracle, specs):
    import torch
    dev, ref = [], []
    for fmt, w, h, seed, fills in specs:
        s0 = Surface.init(fmt, w, h)
        if fmt in ("rgba", "argb"):
            s0.data[:] = premultiplied_background(np.random.default_rng(seed), w, h)
        dev.append(s0.to_device("cuda"))
        r = Surface.init(fmt, w, h)
        r.data[:] = s0.data
        for pat, nodes, opts in fills:
            assert oracle.fill(r, pat, nodes, opts) == abi.OK
        ref.append(r)
    return dev, ref


@pytest.mark.parametrize("seed", range(6))
def test_many_surfaces(oracle, seed):
    """fill_jobs with a few short fills per surface: the one-upload path
    over several surfaces (the multi-surface rasteriser), then the same jobs
    with a large off-surface fill added to the last one (the pipeline)."""
    import torch
    rng = np.random.default_rng(1300 + seed)
    specs = []
    for j in range(int(rng.integers(2, 7))):
        w, h = int(rng.integers(8, 260)), int(rng.integers(8, 200))
        fills = []
        for k in range(int(rng.integers(1, 3))):
            nodes = random_path(rng, w, h, side_lo=4.0, side_hi=float(min(40, max(w, h))), seg_hi=5)
            op = str(rng.choice(["src_over", "src_over", "multiply", "src_in", "xor", "hue"]))
            fills.append((Pattern.from_pixel(Pixel.rgba(int(rng.integers(0, 120)), 90, 40, 200)), nodes,
                          FillOptions(operator=op, fill_rule=str(rng.choice(["non_zero", "even_odd"])))))
        specs.append((str(rng.choice(["rgba", "rgb", "alpha8"])), w, h, seed * 31 + j, fills))
    from z2d_gb300.native import default_context
    ctx = default_context()
    for big in (False, True):
        dev, ref = _dev_jobs(oracle, specs)
        jobs = [(d, list(sp[4])) for d, sp in zip(dev, specs)]
        if big:
            jobs[-1][1].append((Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4)), _off_surface(), FillOptions()))
        n0 = ctx.launch_count
        painter.fill_jobs(jobs, ctx=ctx)
        torch.cuda.synchronize()
        assert (ctx.launch_count - n0 <= 1) == (not big), "the call did not take the intended path"
        for k, (d, r) in enumerate(zip(dev, ref)):
            assert np.array_equal(d.to_host().numpy(), r.numpy()), f"job {k} ({'pipeline' if big else 'one upload'})"
