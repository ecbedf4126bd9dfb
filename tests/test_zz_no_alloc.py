"""z2dgpu_composite_noalloc against z2dgpu_composite, through the C ABI.

The allocation-free entry point runs the same compositor kernels with its
gradient descriptors in a fixed device array, so results must match the
context-based entry point exactly (tolerance 0), including on the second
of two calls in a row that reuse that array with different gradients.
"""
import numpy as np
import pytest

from z2d_gb300 import abi
from z2d_gb300.compositor import SurfaceCompositor, run_noalloc
from z2d_gb300.native import Z2DError, default_context
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, Gradient, Operation, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background

pytestmark = pytest.mark.gpu

TOL = 0  # same kernels, same descriptors: bit-exact


def _grad(kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "linear":
        g = Gradient.linear(3, 5, 150, 90)
    elif kind == "radial":
        g = Gradient.radial(70, 40, 4, 60, 50, 90, method="srgb")
    else:
        g = Gradient.conic(80, 45, 1.3, method="hsl")
    for off in sorted(rng.uniform(0, 1, 4)):
        c = rng.uniform(0, 1, 4)
        g.add_stop(float(off), Color.rgb(*map(float, c)))
    return g


def _bg(fmt, w, h, seed):
    rng = np.random.default_rng(seed)
    s = Surface.init(fmt, w, h)
    if fmt == "rgba":
        s.data[:] = premultiplied_background(rng, w, h)
    elif fmt == "rgb":
        d = rng.integers(0, 256, size=s.data.size, dtype=np.uint8)
        d.reshape(-1, 4)[:, 3] = 0
        s.data[:] = d
    else:
        s.data[:] = rng.integers(0, 256, size=s.data.size, dtype=np.uint8)
    return s


def _calls(w, h):
    """Two consecutive batches with different gradients (4 gradient params
    in the first, the most one call can hold)."""
    mask = Surface.init("alpha8", w, h)
    mask.data[:] = np.random.default_rng(7).integers(0, 256, size=mask.data.size, dtype=np.uint8)
    src = _bg("rgba", w - 9, h - 5, 12)
    first = ([Operation("dst_in", dst=Pattern.from_gradient(_grad("linear", 1)),
                        src=Pattern.dither("blue_noise", _grad("radial", 2), 8)),
              Operation("src_over", dst=Pattern.from_gradient(_grad("conic", 3)),
                        src=Pattern.dither("bayer", _grad("linear", 4), 4))], 0, 0, "float")
    second = ([Operation("dst_in", dst=Pattern.from_gradient(_grad("radial", 5)), src=mask),
               Operation("multiply")], 0, 0, "integer")
    third = ([Operation("src_over", src=src)], 6, 3, "integer")
    fourth = ([Operation("hard_light", src=Pattern.dither("blue_noise", _grad("conic", 6), 8))], 0, 0, "integer")
    return [first, second, third, fourth]


def _dev(s):
    return s.to_device("cuda")


def _cmp(a, b, what):
    x = a.to_host().numpy().astype(np.int16)
    y = b.to_host().numpy().astype(np.int16)
    d = np.abs(x - y)
    assert int(d.max(initial=0)) <= TOL, f"{what}: {int((d > 0).sum())} bytes differ"


def _dev_calls(w, h):
    return [([Operation(o.operator, dst=_dev(o.dst) if isinstance(o.dst, Surface) else o.dst,
                        src=_dev(o.src) if isinstance(o.src, Surface) else o.src) for o in ops], x, y, prec)
            for ops, x, y, prec in _calls(w, h)]


@pytest.mark.parametrize("fmt", ["rgba", "rgb", "alpha8", "alpha2"])
def test_noalloc_matches_composite(fmt):
    """Each call, checked after it completes."""
    torch = pytest.importorskip("torch")
    w, h = 157, 93
    ctx = default_context()
    a, b = _dev(_bg(fmt, w, h, 21)), _dev(_bg(fmt, w, h, 21))
    stream = torch.cuda.current_stream().cuda_stream
    for i, (ops, x, y, prec) in enumerate(_dev_calls(w, h)):
        run_noalloc(a, x, y, ops, prec, device=0, stream=stream)
        SurfaceCompositor.run(b, x, y, ops, prec, ctx=ctx)
        torch.cuda.synchronize()
        _cmp(a, b, f"{fmt} call {i}")


@pytest.mark.parametrize("fmt", ["rgba", "alpha8"])
def test_noalloc_calls_queued_on_one_stream(fmt):
    """All four calls queued back to back on one stream, one synchronisation
    at the end: each call rewrites the shared descriptor array while the
    previous call's kernels may not have run yet, which stream order makes
    safe.  The final surface equals the context path's after the same calls."""
    torch = pytest.importorskip("torch")
    w, h = 157, 93
    ctx = default_context()
    a, b = _dev(_bg(fmt, w, h, 31)), _dev(_bg(fmt, w, h, 31))
    calls = _dev_calls(w, h)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    for ops, x, y, prec in calls:
        run_noalloc(a, x, y, ops, prec, device=0, stream=s.cuda_stream)
    s.synchronize()
    for ops, x, y, prec in calls:
        SurfaceCompositor.run(b, x, y, ops, prec, ctx=ctx)
    torch.cuda.synchronize()
    _cmp(a, b, f"{fmt} after four queued calls")


def test_noalloc_rejects_gradients_while_capturing():
    """A call with a gradient param on a capturing stream is refused before
    it queues anything (its descriptors would be copied from memory that
    does not outlive the call); the capture itself stays valid."""
    torch = pytest.importorskip("torch")
    w, h = 32, 16
    a = _dev(_bg("rgba", w, h, 3))
    ops = [Operation("src_over", src=Pattern.from_gradient(_grad("linear", 9)))]
    s = torch.cuda.Stream()
    run_noalloc(a, 0, 0, ops, device=0, stream=s.cuda_stream)  # first call on the device: outside any capture
    s.synchronize()
    x = torch.zeros(16, device="cuda")
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.graph(g, stream=s):
        try:
            run_noalloc(a, 0, 0, ops, device=0, stream=s.cuda_stream)
        except Z2DError as e:
            err = e
        x.add_(1)
    assert err is not None and err.code == abi.ERR_INVALID_ARGUMENT
    g.replay()
    torch.cuda.synchronize()
    assert float(x.sum()) == 16.0


def test_noalloc_rejects():
    pytest.importorskip("torch")
    w, h = 16, 8
    a = _dev(_bg("rgba", w, h, 1))
    px = Pattern.from_pixel(Pixel.rgba(10, 20, 30, 40))
    with pytest.raises(Z2DError) as e:
        run_noalloc(a, 0, 0, [Operation("src_over", src=px)] * 3)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    with pytest.raises(Z2DError) as e:
        run_noalloc(_bg("rgba", w, h, 1), 0, 0, [Operation("src_over", src=px)])
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    with pytest.raises(Z2DError) as e:
        run_noalloc(a, 0, 0, [Operation("src_over", src=_bg("rgba", w, h, 2))])
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
