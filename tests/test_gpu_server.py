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
