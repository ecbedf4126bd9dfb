"""Gradient offsets of the kernels against the oracle's f64 evaluation.

The kernels evaluate Gradient.getOffset (gradient.zig:239-243, 349-372,
605-648, 731-741) on double-word floats with an error bound and run the f64
code only where the bound leaves the f32 rounding (or one of the code's
comparisons) undecided.  Each case compares every offset of a pixel block
with the oracle's, bit for bit, and checks that the f64 fallback stays rare
where the geometry is ordinary.  The cases aim at what the bound must get
right: offsets that land exactly on floats and just beside f32 rounding
midpoints (scaled axis-aligned gradients), the clamps at 0 and 1, radial
gradients with a = 0, both roots, no root, concentric circles and a focal
point outside the outer circle, the conic branch cut on the centre's row
and the wrap at the start angle, transformed gradients, negative pixel
coordinates, and constants outside the fast path's range.
"""
import math

import numpy as np
import pytest

from z2d_gb300.native import Context
from z2d_gb300.types import Color, Gradient

pytestmark = pytest.mark.gpu

X0, Y0, W, H = -40, -24, 384, 256


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def _stops(g):
    g.add_stop(0.0, Color.rgb(1, 0, 0, 1)).add_stop(1.0, Color.rgb(0, 0, 1, 1))
    return g


def _check(ctx, oracle, g, what, max_slow=None, box=(X0, Y0, W, H)):
    x0, y0, w, h = box
    got, n_slow = ctx.gradient_offsets(g, x0, y0, w, h)
    want = oracle.gradient_offsets(g, x0, y0, w, h)
    bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
    if bad.size:
        j, i = divmod(int(bad[0]), w)
        pytest.fail(f"{what}: {bad.size} offsets differ; first at pixel ({x0 + i}, {y0 + j}): "
                    f"kernel {got.flat[bad[0]]!r} oracle {want.flat[bad[0]]!r}")
    if max_slow is not None:
        assert n_slow <= max_slow * w * h, f"{what}: {n_slow} of {w * h} offsets took the f64 code"
    return n_slow


def _random_tf(rng):
    a = rng.uniform(-math.pi, math.pi)
    sx, sy = rng.uniform(0.3, 3.0, 2)
    sh = rng.uniform(-0.5, 0.5)
    c, s = math.cos(a), math.sin(a)
    return (c * sx, s * sx + sh, -s * sy, c * sy, rng.uniform(-200, 200), rng.uniform(-200, 200))


@pytest.mark.parametrize("seed", range(12))
def test_linear_random(ctx, oracle, seed):
    rng = np.random.default_rng(100 + seed)
    for k in range(4):
        x0, y0, x1, y1 = rng.uniform(-200, 600, 4)
        g = _stops(Gradient.linear(x0, y0, x1, y1))
        if k & 1:
            g.set_transformation(_random_tf(rng))
        _check(ctx, oracle, g, f"linear {seed}/{k}", max_slow=0.01)


@pytest.mark.parametrize("length", [1, 2, 3, 7, 64, 256, 1000, 4096, 1 << 20])
def test_linear_exact_offsets(ctx, oracle, length):
    """Axis-aligned: t = (x + 0.5 - x0) / length, exactly a float for
    power-of-two lengths; the clamps cover the pixels outside."""
    _check(ctx, oracle, _stops(Gradient.linear(0.0, 0.0, float(length), 0.0)), f"x {length}", max_slow=0.01)
    _check(ctx, oracle, _stops(Gradient.linear(3.5, 0.0, 3.5, -float(length))), f"-y {length}", max_slow=0.01)


@pytest.mark.parametrize("k", [20, 22, 23, 24, 25, 26, 28, 30, 34])
def test_linear_near_midpoints(ctx, oracle, k):
    """A scale of 1 + 2^-k puts offsets within about 2^-k of values that are
    floats or f32 midpoints: the rounding direction there is what the bound
    has to decide (or leave to the f64 code)."""
    for sign in (1.0, -1.0):
        g = _stops(Gradient.linear(0.0, 0.0, 1024.0, 0.0))
        g.set_transformation((1.0 + sign * 2.0 ** -k, 0.0, 0.0, 1.0, 0.0, 0.0))
        _check(ctx, oracle, g, f"1 {'+-'[sign < 0]} 2^-{k}", box=(0, 0, 1280, 4))


@pytest.mark.parametrize("seed", range(12))
def test_radial_random(ctx, oracle, seed):
    rng = np.random.default_rng(200 + seed)
    for k in range(4):
        ix, iy, ox, oy = rng.uniform(-100, 450, 4)
        ir, orr = rng.uniform(0, 250, 2)
        if k == 2:
            ir = 0.0
        g = _stops(Gradient.radial(ix, iy, ir, ox, oy, orr))
        if k == 3:
            g.set_transformation(_random_tf(rng))
        _check(ctx, oracle, g, f"radial {seed}/{k}", max_slow=0.02)


@pytest.mark.parametrize("geom", [
    (150, 100, 0, 150, 100, 120),      # concentric, inner radius 0
    (150, 100, 30, 150, 100, 120),     # concentric ring
    (150, 100, 120, 150, 100, 30),     # shrinking (dr < 0)
    (100, 100, 10, 130, 100, 40),      # a = 0: focal circle touching the outer one
    (100, 100, 20, 100, 160, 80),      # a = 0, vertical
    (400, 120, 10, 150, 100, 60),      # focal point outside: a cone, two roots, no root
    (-50, -30, 5, 300, 200, 20),       # both outside, small radii
    (150, 100, 0, 150, 100, 0),        # both radii 0: every offset -1
    (150.5, 100.5, 0, 150.5, 100.5, 64),  # centre on a pixel centre
])
def test_radial_cases(ctx, oracle, geom):
    _check(ctx, oracle, _stops(Gradient.radial(*geom)), f"radial {geom}", max_slow=0.05)


@pytest.mark.parametrize("seed", range(8))
def test_conic_random(ctx, oracle, seed):
    rng = np.random.default_rng(300 + seed)
    for k in range(4):
        cx, cy = rng.uniform(-100, 450, 2)
        ang = rng.uniform(-10, 10)
        g = _stops(Gradient.conic(cx, cy, ang))
        if k & 1:
            g.set_transformation(_random_tf(rng))
        _check(ctx, oracle, g, f"conic {seed}/{k}", max_slow=0.01)


@pytest.mark.parametrize("cx,cy", [(150.5, 100.5), (150.0, 100.0), (0.5, 0.5), (-20.5, 60.5)])
@pytest.mark.parametrize("ang", [0.0, math.pi / 2, math.pi, 3 * math.pi / 2, -math.pi, 2 * math.pi, 0.1])
def test_conic_cuts(ctx, oracle, cx, cy, ang):
    """Centres on pixel centres put pixels exactly on the branch cut and the
    axes; angles at multiples of pi / 2 put the wrap on them too."""
    _check(ctx, oracle, _stops(Gradient.conic(cx, cy, ang)), f"conic ({cx}, {cy}) {ang}", max_slow=0.02)


def test_constants_outside_fast_range(ctx, oracle):
    """Constants the double-word path does not take (a gradient of length
    1e-12, so 1 / |d|^2 = 1e24; an inverse scale of 1e-20; an angle of
    1e-300) run on the f64 code alone; large but accepted ones (a scale of
    1e12) overflow the bounds of most pixels, which then take the f64 code
    too."""
    _check(ctx, oracle, _stops(Gradient.linear(10.0, 10.0, 10.0 + 1e-12, 10.0)), "tiny linear")
    for s in (1e20, 1e12):
        g = _stops(Gradient.radial(100, 100, 0, 100, 100, 80))
        g.set_transformation((s, 0.0, 0.0, s, 0.0, 0.0))
        _check(ctx, oracle, g, f"scale {s}")
    _check(ctx, oracle, _stops(Gradient.conic(100.0, 100.0, 1e-300)), "tiny angle")


def test_far_pixels(ctx, oracle):
    """Pixel coordinates beyond 2^22 take the f64 code."""
    g = _stops(Gradient.linear(0.0, 0.0, 8e6, 3e6))
    _check(ctx, oracle, g, "far", box=((1 << 22) - 64, 5, 128, 4))
