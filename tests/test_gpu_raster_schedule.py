"""The persistent rasteriser's schedules (z2dgpu_ctx_set_raster) and their
autotuner.  Warps take (tile, row) items from a device queue, so the order
in which tiles are drawn changes with the schedule; the pixels must not:
every schedule matches the oracle bit for bit, on one surface and on many."""
import json
import os

import numpy as np
import pytest

from z2d_gb300 import abi, painter
from z2d_gb300.native import Context
from z2d_gb300.surface import Surface
from z2d_gb300.workloads import premultiplied_background, random_fills

pytestmark = pytest.mark.gpu

SCHEDULES = [(-1, 0, 1), (-1, 1, 1), (0, 0, 1), (0, 1, 1), (0, 0, 0), (0, 1, 0), (4, 1, 1), (2, 1, 0), (1, 0, 1)]


def _bg(w, h, seed):
    s = Surface.init("rgba", w, h)
    s.data[:] = premultiplied_background(np.random.default_rng(seed), w, h)
    return s


@pytest.fixture(scope="module")
def one_surface(oracle):
    w, h = 700, 420
    fills = random_fills(seed=41, n=120, w=w, h=h, side_lo=8, side_hi=500, seg_lo=3, seg_hi=40)
    ref = _bg(w, h, 3)
    for pat, nodes, opts in fills:
        assert oracle.fill(ref, pat, nodes, opts) == abi.OK
    return w, h, fills, ref.numpy()


@pytest.mark.parametrize("ctas,order,tile_items", SCHEDULES)
def test_schedule_one_surface(one_surface, ctas, order, tile_items):
    w, h, fills, ref = one_surface
    ctx = Context(0)
    ctx.set_raster(ctas, order, tile_items)
    s = _bg(w, h, 3)
    painter.fill_batch(s, fills, ctx=ctx)
    got = s.numpy()
    assert np.array_equal(got, ref), f"{int((got != ref).any(-1).sum())} pixels differ"
    ctx.close()


@pytest.mark.parametrize("ctas,order,tile_items", SCHEDULES)
def test_schedule_many_surfaces(oracle, ctas, order, tile_items):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    specs = []
    for j in range(30):
        w, h = int(rng.integers(16, 400)), int(rng.integers(16, 300))
        specs.append((w, h, random_fills(seed=500 + j, n=int(rng.integers(1, 20)), w=w, h=h, side_lo=4,
                                         side_hi=min(w, h), seg_lo=3, seg_hi=20)))
    ctx = Context(0)
    ctx.set_raster(ctas, order, tile_items)
    dev = [_bg(w, h, 60 + j).to_device("cuda") for j, (w, h, _) in enumerate(specs)]
    painter.fill_jobs([(d, f) for d, (_, _, f) in zip(dev, specs)], ctx=ctx)
    torch.cuda.synchronize()
    for j, (w, h, fills) in enumerate(specs):
        ref = _bg(w, h, 60 + j)
        for pat, nodes, opts in fills:
            assert oracle.fill(ref, pat, nodes, opts) == abi.OK
        assert np.array_equal(dev[j].to_host().numpy(), ref.numpy()), f"job {j}"
    ctx.close()


def test_autotuner_decides_and_caches(one_surface):
    """Unforced, the first passes of a kind time the candidate schedules;
    then the tuner has decided, the pixels are still exact, and the choice
    is in the JSON cache."""
    w, h, fills, ref = one_surface
    ctx = Context(0)
    state = None
    for _ in range(8):
        s = _bg(w, h, 3)
        painter.fill_batch(s, fills, ctx=ctx)
        assert np.array_equal(s.numpy(), ref)
        state = ctx.raster_tuning()
        if state["decided"] != 0:
            break
    ctx.close()
    if state["decided"] == -1:
        pytest.skip("autotuning is off (Z2D_TUNE=off)")
    assert state["decided"] == 1, state
    path = os.environ.get("Z2D_TUNE_FILE")
    if path and os.path.exists(path):
        lines = [json.loads(x) for x in open(path) if x.strip()]
        assert lines and all({"multi", "tiles", "load", "ctas", "order", "cta_items", "ms"} <= set(d) for d in lines)


def test_set_raster_rejects():
    from z2d_gb300.native import Z2DError
    ctx = Context(0)
    with pytest.raises(Z2DError):
        ctx.set_raster(4, 2)
    with pytest.raises(Z2DError):
        ctx.set_raster(4, 0, 2)
    with pytest.raises(Z2DError):
        ctx.set_raster(-3, 0)
    ctx.set_raster(-2, 0)  # back to the tuner
    ctx.close()
