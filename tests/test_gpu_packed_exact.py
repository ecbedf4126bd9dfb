"""Packed alpha surfaces (alpha4 / alpha2 / alpha1) in device buffers of
z2d's exact length, ceil(w * h * bits / 8) bytes, that is not a whole number
of 32-bit words.  The pixels are updated with word atomics, so the library
draws such a surface on a padded copy; here every surface sits at the start
of a larger buffer whose trailing guard bytes must come out unchanged, and
the pixels must equal the oracle's, through every drawing entry point."""
import numpy as np
import pytest

from backends import StrokeOracle
from z2d_gb300 import abi, compositor, painter
from z2d_gb300.surface import Surface
from z2d_gb300.types import FillOptions, Operation, Pattern, Pixel, StrokeOptions
from z2d_gb300.workloads import random_fills, random_path

pytestmark = pytest.mark.gpu

GUARD = 64
# (format, w, h) whose byte length is 1, 2 or 3 past a multiple of 4
CASES = [("alpha1", 7, 5), ("alpha1", 61, 3), ("alpha2", 11, 5), ("alpha2", 29, 9), ("alpha4", 7, 3), ("alpha4", 35, 9)]


def _exact(fmt, w, h, seed):
    """A device surface of exactly z2d's length, followed by guard bytes."""
    torch = pytest.importorskip("torch")
    n = abi.surface_bytes(abi.FORMAT_NAMES.index(fmt), w, h)
    assert n % 4 != 0
    host = np.random.default_rng(seed).integers(0, 256, n + GUARD, dtype=np.uint8)
    buf = torch.from_numpy(host.copy()).to("cuda")
    ref = Surface(fmt, w, h, host[:n].copy())
    return Surface(fmt, w, h, buf[:n]), buf, host[n:].copy(), ref


def _check(dev, buf, guard, ref, what):
    import torch
    torch.cuda.synchronize()
    n = abi.surface_bytes(dev.format, dev.width, dev.height)
    out = buf.cpu().numpy()
    assert np.array_equal(out[n:], guard), f"{what}: bytes past the surface changed"
    assert np.array_equal(out[:n], ref.numpy()), f"{what}: pixels differ from the oracle"


@pytest.mark.parametrize("fmt,w,h", CASES)
def test_fill_and_batch(oracle, fmt, w, h):
    fills = random_fills(seed=w * h, n=6, w=w, h=h, side_lo=2, side_hi=max(3, min(w, h)), seg_lo=3, seg_hi=12)
    dev, buf, guard, ref = _exact(fmt, w, h, 1)
    pat, nodes, opts = fills[0]
    painter.fill(dev, pat, nodes, opts)
    assert oracle.fill(ref, pat, nodes, opts) == abi.OK
    painter.fill_batch(dev, fills[1:])
    for pat, nodes, opts in fills[1:]:
        assert oracle.fill(ref, pat, nodes, opts) == abi.OK
    _check(dev, buf, guard, ref, f"fill {fmt} {w}x{h}")


@pytest.mark.parametrize("fmt,w,h", CASES)
def test_stroke_and_hairline(oracle, fmt, w, h):
    rng = np.random.default_rng(w + h)
    dev, buf, guard, ref = _exact(fmt, w, h, 2)
    so = StrokeOracle(oracle)
    pat = Pattern.from_pixel(Pixel.rgba(200, 100, 50, 220))
    for hair in (False, True):
        nodes = random_path(rng, w, h, 2, max(3, min(w, h)), 3, 8)
        opts = StrokeOptions(line_width=2.5, hairline=hair)
        painter.stroke(dev, pat, nodes, opts)
        assert so.stroke(ref, pat, nodes, opts) == abi.OK
    _check(dev, buf, guard, ref, f"stroke {fmt} {w}x{h}")


def test_jobs_and_draw_jobs(oracle):
    """Many exact-length packed surfaces in one pass, fills, strokes and
    hairlines mixed."""
    rng = np.random.default_rng(4)
    so = StrokeOracle(oracle)
    items, jobs = [], []
    for k, (fmt, w, h) in enumerate(CASES * 2):
        dev, buf, guard, ref = _exact(fmt, w, h, 10 + k)
        ops = []
        for i in range(4):
            pat = Pattern.from_pixel(Pixel.rgba(30 * i, 60, 90, 200))
            nodes = random_path(rng, w, h, 2, max(3, min(w, h)), 3, 10)
            if i % 2 == 0:
                ops.append(("fill", pat, nodes, FillOptions()))
            else:
                ops.append(("stroke", pat, nodes, StrokeOptions(line_width=1.5 + i, hairline=(i == 3))))
        for kind, pat, nodes, o in ops:
            rc = oracle.fill(ref, pat, nodes, o) if kind == "fill" else so.stroke(ref, pat, nodes, o)
            assert rc == abi.OK
        items.append((dev, buf, guard, ref))
        jobs.append((dev, ops))
    painter.draw_jobs(jobs)
    for k, (dev, buf, guard, ref) in enumerate(items):
        _check(dev, buf, guard, ref, f"job {k}")


@pytest.mark.parametrize("fmt,w,h", CASES)
def test_composite(oracle, fmt, w, h):
    dev, buf, guard, ref = _exact(fmt, w, h, 3)
    mask = Surface.init("alpha8", w, h)
    mask.data[:] = np.random.default_rng(5).integers(0, 256, mask.data.size, dtype=np.uint8)
    ops = [Operation("dst_in", dst=Pattern.from_pixel(Pixel.rgba(10, 20, 30, 180)), src=mask.to_device("cuda")),
           Operation("xor")]
    compositor.SurfaceCompositor.run(dev, 0, 0, ops)
    assert oracle.composite(ref, 0, 0, [Operation("dst_in", dst=ops[0].dst, src=mask), Operation("xor")]) == abi.OK
    _check(dev, buf, guard, ref, f"composite {fmt} {w}x{h}")
