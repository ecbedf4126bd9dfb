"""The serving queue (z2dgpu_server_*): every request's result equals the
same fills drawn alone, whatever batch it lands in; requests on one surface
keep their submission order; a failing request fails alone."""
import threading

import numpy as np
import pytest

from z2d_gb300 import abi
from z2d_gb300.native import Z2DError
from z2d_gb300.server import Server
from z2d_gb300.surface import Surface
from z2d_gb300.types import FillOptions, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background, random_fills

pytestmark = pytest.mark.gpu


def _bg(w, h, seed):
    s = Surface.init("rgba", w, h)
    s.data[:] = premultiplied_background(np.random.default_rng(seed), w, h)
    return s


def _requests(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = int(rng.integers(8, 200)), int(rng.integers(8, 160))
        fills = random_fills(seed=seed * 1000 + i, n=int(rng.integers(1, 8)), w=w, h=h, side_lo=2,
                             side_hi=max(3, min(w, h)), seg_lo=3, seg_hi=12)
        for k, (_, _, o) in enumerate(fills):
            o.anti_aliasing = ("default", "none", "supersample_4x")[(i + k) % 3]
        out.append((w, h, fills))
    return out


@pytest.mark.parametrize("max_batch,max_wait", [(1, 0), (64, 500), (1000, 5000)])
def test_server_matches_oracle(oracle, max_batch, max_wait):
    torch = pytest.importorskip("torch")
    reqs = _requests(60, seed=max_batch)
    # 12 surfaces, 5 requests each, interleaved: order per surface matters
    surf_specs = [(reqs[i][0], reqs[i][1]) for i in range(12)]
    dev = [_bg(w, h, 50 + k).to_device("cuda") for k, (w, h) in enumerate(surf_specs)]
    ref = [_bg(w, h, 50 + k) for k, (w, h) in enumerate(surf_specs)]
    with Server(max_batch_jobs=max_batch, max_wait_us=max_wait) as srv:
        tickets = []
        for i, (_, _, fills) in enumerate(reqs):
            k = i % 12
            tickets.append(srv.submit(dev[k], fills))
            for pat, nodes, opts in fills:
                assert oracle.fill(ref[k], pat, nodes, opts) == abi.OK
        for t in tickets:
            assert srv.wait(t) >= 0.0
        batches, done, _ = srv.stats()
        assert done == len(reqs) and batches >= 1
    torch.cuda.synchronize()
    for k in range(12):
        a, b = dev[k].to_host().numpy(), ref[k].numpy()
        assert np.array_equal(a, b), f"surface {k}: {int((a != b).sum())} bytes differ"


def test_server_many_threads(oracle):
    torch = pytest.importorskip("torch")
    reqs = _requests(80, seed=7)
    dev = [_bg(w, h, 300 + i).to_device("cuda") for i, (w, h, _) in enumerate(reqs)]
    with Server(max_batch_jobs=32, max_wait_us=300) as srv:
        errors = []

        def client(idx):
            try:
                ts = [srv.submit(dev[i], reqs[i][2]) for i in idx]
                for t in ts:
                    srv.wait(t)
            except Exception as e:  # reported below
                errors.append(e)

        th = [threading.Thread(target=client, args=(list(range(j, 80, 4)),)) for j in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errors
    torch.cuda.synchronize()
    for i, (w, h, fills) in enumerate(reqs):
        r = _bg(w, h, 300 + i)
        for pat, nodes, opts in fills:
            assert oracle.fill(r, pat, nodes, opts) == abi.OK
        assert np.array_equal(dev[i].to_host().numpy(), r.numpy()), f"request {i}"


def test_server_failing_request_fails_alone(oracle):
    torch = pytest.importorskip("torch")
    good = _requests(6, seed=11)
    dev = [_bg(w, h, 400 + i).to_device("cuda") for i, (w, h, _) in enumerate(good)]
    bad_surface = _bg(20, 20, 1).to_device("cuda")
    open_path = [(abi.MOVE_TO, 1, 1, 0, 0, 0, 0), (abi.LINE_TO, 5, 5, 0, 0, 0, 0)]
    with Server(max_batch_jobs=64, max_wait_us=20000) as srv:
        ts = [srv.submit(dev[i], good[i][2]) for i in range(3)]
        tb = srv.submit(bad_surface, [(Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4)), open_path, FillOptions())])
        ts += [srv.submit(dev[i], good[i][2]) for i in range(3, 6)]
        with pytest.raises(Z2DError) as e:
            srv.wait(tb)
        assert e.value.code == abi.ERR_PATH_NOT_CLOSED
        for t in ts:
            srv.wait(t)
    torch.cuda.synchronize()
    for i, (w, h, fills) in enumerate(good):
        r = _bg(w, h, 400 + i)
        for pat, nodes, opts in fills:
            assert oracle.fill(r, pat, nodes, opts) == abi.OK
        assert np.array_equal(dev[i].to_host().numpy(), r.numpy())


def test_server_rejects_host_surface():
    pytest.importorskip("torch")
    with Server() as srv:
        with pytest.raises(Z2DError) as e:
            srv.submit(_bg(8, 8, 1), random_fills(seed=1, n=1, w=8, h=8, side_lo=2, side_hi=6, seg_lo=3, seg_hi=4))
        assert e.value.code == abi.ERR_INVALID_ARGUMENT


def _pool_requests(n, seed):
    """Requests on pool surfaces: several formats, random sizes, half of
    them starting from a seeded background, half cleared."""
    rng = np.random.default_rng(seed)
    fmts = ["rgba", "rgba", "rgb", "alpha8", "alpha4", "alpha1"]
    out = []
    for i in range(n):
        fmt = fmts[i % len(fmts)]
        w, h = int(rng.integers(1, 140)), int(rng.integers(1, 120))
        fills = random_fills(seed=seed * 1000 + i, n=int(rng.integers(0, 6)), w=w, h=h, side_lo=2,
                             side_hi=max(3, min(w, h)), seg_lo=3, seg_hi=12)
        for k, (_, _, o) in enumerate(fills):
            o.anti_aliasing = ("default", "none", "supersample_4x")[(i + k) % 3]
        init = None
        if i % 2:
            s = Surface.init(fmt, w, h)
            s.data[:] = rng.integers(0, 256, s.data.size, dtype=np.uint8)
            if fmt == "rgba":
                s.data[:] = premultiplied_background(rng, w, h)
            init = s.data.copy()
        out.append((fmt, w, h, fills, init))
    return out


def _drawn_alone(oracle, fmt, w, h, fills, init):
    s = Surface.init(fmt, w, h)
    if init is not None:
        s.data[:] = init
    for pat, nodes, opts in fills:
        assert oracle.fill(s, pat, nodes, opts) == abi.OK
    return s.numpy()


@pytest.mark.parametrize("lanes", [1, 3])
def test_server_pool_surfaces_match_drawn_alone(oracle, lanes):
    """Every request on a pool surface, drawn in batches that overlap on the
    GPU, reads back exactly what drawing it alone gives."""
    pytest.importorskip("torch")
    reqs = _pool_requests(90, seed=20 + lanes)
    outs = [np.zeros(abi.surface_bytes(abi.FORMAT_NAMES.index(f), w, h), np.uint8) for f, w, h, _, _ in reqs]
    with Server(max_batch_jobs=16, max_wait_us=100, lanes=lanes, pool_bytes=64 << 20) as srv:
        ts = [srv.submit_new(f, w, h, fills, init=init, out=outs[i]) for i, (f, w, h, fills, init) in enumerate(reqs)]
        for t in ts:
            srv.wait(t)
        info = srv.info()
    assert info["requests"] == len(reqs) and info["lanes"] == lanes
    assert info["pool_peak_bytes"] <= info["pool_bytes"]
    for i, (f, w, h, fills, init) in enumerate(reqs):
        ref = _drawn_alone(oracle, f, w, h, fills, init)
        assert np.array_equal(outs[i], ref), f"request {i} ({f} {w}x{h}): {int((outs[i] != ref).sum())} bytes differ"


def test_server_batches_overlap_on_the_gpu(oracle):
    """With two lanes and a backlog of requests, a second batch starts while
    the first is still being drawn; results are still those drawn alone."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(240):
        w, h = int(rng.integers(200, 400)), int(rng.integers(150, 300))
        reqs.append(("rgba", w, h, random_fills(seed=9000 + i, n=int(rng.integers(4, 12)), w=w, h=h, side_lo=8,
                                                side_hi=min(w, h), seg_lo=3, seg_hi=40), None))
    outs = [np.zeros(w * h * 4, np.uint8) for _, w, h, _, _ in reqs]
    with Server(max_batch_jobs=24, max_wait_us=0, lanes=2, pool_bytes=256 << 20) as srv:
        ts = [srv.submit_new(f, w, h, fills, out=outs[i]) for i, (f, w, h, fills, _) in enumerate(reqs)]
        for t in ts:
            srv.wait(t)
        info = srv.info()
    assert info["batches"] >= 2
    assert info["max_inflight"] >= 2, info
    for i in range(0, len(reqs), 7):
        f, w, h, fills, init = reqs[i]
        assert np.array_equal(outs[i], _drawn_alone(oracle, f, w, h, fills, init)), f"request {i}"


def test_server_pool_admission_waits_for_space(oracle):
    """A pool that holds only a few surfaces at a time: requests wait for
    space (deferred admissions), the pool's high-water mark stays within
    it, and every result is still exact."""
    pytest.importorskip("torch")
    reqs = [("rgba", 64, 64, random_fills(seed=7000 + i, n=3, w=64, h=64, side_lo=4, side_hi=60, seg_lo=3,
                                          seg_hi=20), None) for i in range(120)]
    outs = [np.zeros(64 * 64 * 4, np.uint8) for _ in reqs]
    pool = 4 * 64 * 64 * 4  # room for four surfaces
    with Server(max_batch_jobs=32, max_wait_us=0, lanes=2, pool_bytes=pool) as srv:
        ts = [srv.submit_new(f, w, h, fills, out=outs[i]) for i, (f, w, h, fills, _) in enumerate(reqs)]
        for t in ts:
            srv.wait(t)
        info = srv.info()
    assert info["pool_bytes"] == pool
    assert info["pool_peak_bytes"] <= pool
    assert info["deferred"] > 0
    for i, (f, w, h, fills, init) in enumerate(reqs):
        assert np.array_equal(outs[i], _drawn_alone(oracle, f, w, h, fills, init)), f"request {i}"


def test_server_pool_rejections():
    pytest.importorskip("torch")
    fills = random_fills(seed=1, n=1, w=8, h=8, side_lo=2, side_hi=6, seg_lo=3, seg_hi=4)
    with Server(pool_bytes=1 << 16) as srv:
        with pytest.raises(Z2DError) as e:
            srv.submit_new("rgba", 512, 512, fills)  # 1 MiB surface, 64 KiB pool
        assert e.value.code == abi.ERR_OUT_OF_MEMORY
    with Server() as srv:  # no pool
        with pytest.raises(Z2DError) as e:
            srv.submit_new("rgba", 8, 8, fills)
        assert e.value.code == abi.ERR_INVALID_STATE
