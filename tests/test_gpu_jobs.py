"""Multi-surface batches (z2dgpu_fill_jobs) against the oracle: every job's
surface must equal painter.fill applied to it command by command."""
import numpy as np
import pytest

from z2d_gb300 import abi, painter
from z2d_gb300.native import Z2DError
from z2d_gb300.surface import Surface
from z2d_gb300.types import Color, FillOptions, Gradient, Pattern, Pixel
from z2d_gb300.workloads import batched_jobs, job_fills, premultiplied_background, random_fills

pytestmark = pytest.mark.gpu


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


def _run(oracle, specs):
    """specs: (fmt, w, h, seed, fills) per job; returns (gpu, oracle) surfaces."""
    dev, ref = [], []
    for fmt, w, h, seed, fills in specs:
        dev.append(_bg(fmt, w, h, seed).to_device("cuda"))
        r = _bg(fmt, w, h, seed)
        for pat, nodes, opts in fills:
            assert oracle.fill(r, pat, nodes, opts) == abi.OK
        ref.append(r)
    painter.fill_jobs([(d, spec[4]) for d, spec in zip(dev, specs)])
    import torch
    torch.cuda.synchronize()
    return [d.to_host() for d in dev], ref


def _cmp(a, b, what, tol=0):
    d = np.abs(a.numpy().astype(np.int16) - b.numpy().astype(np.int16))
    assert int(d.max(initial=0)) <= tol, f"{what}: {int((d > 0).sum())} bytes differ"


def test_jobs_mixed(oracle):
    pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    fmts = ["rgba", "argb", "rgb", "alpha8", "alpha4", "alpha2", "alpha1", "xrgb"]
    aas = ["default", "none", "supersample_4x"]
    ops = ["src_over", "src_over", "multiply", "src_in", "clear", "xor", "color_burn"]
    g = Gradient.linear(0, 0, 200, 150)
    g.add_stop(0.0, Color.rgb(1, 0, 0, 1))
    g.add_stop(1.0, Color.rgb(0, 0, 1, 0.5))
    specs = []
    for j in range(40):
        w, h = int(rng.integers(1, 300)), int(rng.integers(1, 260))
        n = int(rng.integers(0, 12))
        fills = random_fills(seed=1000 + j, n=n, w=w, h=h, side_lo=2, side_hi=max(3, min(w, h)), seg_lo=3, seg_hi=16)
        for i, (pat, nodes, opts) in enumerate(fills):
            opts.anti_aliasing = aas[(i + j) % 3]
            opts.operator = ops[(i * 3 + j) % len(ops)]
            if (i + j) % 5 == 0:
                fills[i] = (Pattern.from_gradient(g), nodes, opts)
        specs.append((fmts[j % len(fmts)], w, h, j, fills))
    got, ref = _run(oracle, specs)
    for j, (a, b) in enumerate(zip(got, ref)):
        _cmp(a, b, f"job {j} ({specs[j][0]} {specs[j][1]}x{specs[j][2]})")


def test_jobs_batched_workload_slice(oracle):
    pytest.importorskip("torch")
    jobs = batched_jobs(seed=77, n_jobs=24, side_lo=16, side_hi=512, paths_lo=1, paths_hi=40)
    specs = [("rgba", jb[0], jb[1], 100 + j, job_fills(jb)) for j, jb in enumerate(jobs)]
    got, ref = _run(oracle, specs)
    for j, (a, b) in enumerate(zip(got, ref)):
        _cmp(a, b, f"job {j}")


def test_jobs_single_equals_batch(oracle):
    pytest.importorskip("torch")
    w, h = 300, 200
    fills = random_fills(seed=9, n=60, w=w, h=h, side_lo=4, side_hi=250, seg_lo=3, seg_hi=30)
    a = _bg("rgba", w, h, 1).to_device("cuda")
    b = _bg("rgba", w, h, 1).to_device("cuda")
    painter.fill_jobs([(a, fills)])
    painter.fill_batch(b, fills)
    import torch
    torch.cuda.synchronize()
    _cmp(a.to_host(), b.to_host(), "single job vs batch")


def test_jobs_empty_and_offsurface(oracle):
    pytest.importorskip("torch")
    far = [(Pattern.from_pixel(Pixel.rgba(10, 20, 30, 40)),
            [(abi.MOVE_TO, 900, 900, 0, 0, 0, 0), (abi.LINE_TO, 950, 900, 0, 0, 0, 0),
             (abi.LINE_TO, 950, 990, 0, 0, 0, 0), (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)], FillOptions())]
    specs = [("rgba", 50, 40, 1, []), ("rgba", 60, 30, 2, far), ("alpha8", 33, 17, 3,
             random_fills(seed=4, n=5, w=33, h=17, side_lo=2, side_hi=16, seg_lo=3, seg_hi=8)), ("rgba", 10, 10, 4, [])]
    got, ref = _run(oracle, specs)
    for j, (a, b) in enumerate(zip(got, ref)):
        _cmp(a, b, f"job {j}")


def test_jobs_errors():
    pytest.importorskip("torch")
    host = _bg("rgba", 8, 8, 1)
    fills = random_fills(seed=1, n=1, w=8, h=8, side_lo=2, side_hi=6, seg_lo=3, seg_hi=4)
    with pytest.raises(Z2DError) as e:
        painter.fill_jobs([(host, fills)])
    assert e.value.code == abi.ERR_INVALID_ARGUMENT


def test_jobs_packed_arrays(oracle):
    """The numpy-packed entry (z2d_gb300.batch) draws what the oracle draws."""
    pytest.importorskip("torch")
    from z2d_gb300.batch import PackedBatch
    jobs = batched_jobs(seed=91, n_jobs=16, side_lo=16, side_hi=400, paths_lo=1, paths_hi=30)
    nodes, offs, cnts, pxs, rules, cmd_off, cmd_cnt = [], [], [], [], [], [], []
    base = ncmd = 0
    for w, h, nd, off, cnt, px, rl in jobs:
        nodes.append(nd)
        offs.append(off + base)
        cnts.append(cnt)
        pxs.append(px)
        rules.append(rl)
        cmd_off.append(ncmd)
        cmd_cnt.append(len(off))
        base += len(nd)
        ncmd += len(off)
    pb = PackedBatch(np.concatenate(nodes), np.concatenate(offs), np.concatenate(cnts), np.concatenate(pxs),
                     np.concatenate(rules))
    dev = [_bg("rgba", jb[0], jb[1], 200 + j).to_device("cuda") for j, jb in enumerate(jobs)]
    pb.set_jobs(dev, cmd_off, cmd_cnt)
    pb.fill_jobs()
    import torch
    torch.cuda.synchronize()
    for j, jb in enumerate(jobs):
        ref = _bg("rgba", jb[0], jb[1], 200 + j)
        for pat, nd, opts in job_fills(jb):
            assert oracle.fill(ref, pat, nd, opts) == abi.OK
        _cmp(dev[j].to_host(), ref, f"job {j}")
