"""Batch preparation: commands whose node ranges come in any order or leave
nodes unclaimed, overlapping ranges, and the error of the first failing
command of a large batch (prepared on host threads)."""
import ctypes as C

import numpy as np
import pytest

from z2d_gb300 import abi, painter
from z2d_gb300.native import Z2DError
from z2d_gb300.surface import Surface
from z2d_gb300.types import FillOptions, Pattern, Pixel
from z2d_gb300.workloads import premultiplied_background, random_fills

pytestmark = pytest.mark.gpu


def _bg(w, h, seed):
    s = Surface.init("rgba", w, h)
    s.data[:] = premultiplied_background(np.random.default_rng(seed), w, h)
    return s


def _cmds(fills, offsets):
    """A z2d_fill_cmd array: fill i reads its nodes at offsets[i]."""
    keep = []
    cmds = (abi.z2d_fill_cmd * len(fills))()
    for i, (pat, n, opts) in enumerate(fills):
        cmds[i].pattern = C.pointer(pat.to_abi(keep))
        cmds[i].node_offset = offsets[i]
        cmds[i].n_nodes = len(n)
        cmds[i].opts = opts.to_abi()
    return cmds, keep


def _junk(n):
    j = np.zeros(n, dtype=random_fills(0, 1, 8, 8)[0][1].dtype)
    j["tag"] = 7  # not a node tag: must never be read as a path
    j["p"] = np.nan
    return j


@pytest.mark.parametrize("n", [20, 300])
def test_node_ranges_in_any_order_with_gaps(oracle, n):
    w, h = 384, 256
    fills = random_fills(seed=11, n=n, w=w, h=h, side_lo=8, side_hi=200, seg_lo=3, seg_hi=30)
    # the node array holds the paths in reverse order, with unclaimed junk
    # nodes before, between and after them
    parts, offsets, off = [], [0] * n, 0
    for i in reversed(range(n)):
        junk = _junk(1 + i % 3)
        parts += [junk, fills[i][1]]
        off += len(junk)
        offsets[i] = off
        off += len(fills[i][1])
    parts.append(_junk(5))
    nodes = np.ascontiguousarray(np.concatenate(parts))
    cmds, keep = _cmds(fills, offsets)
    a, b = _bg(w, h, 3), _bg(w, h, 3)
    painter.fill_batch_arrays(a, nodes, cmds)
    for pat, nd, opts in fills:
        assert oracle.fill(b, pat, nd, opts) == abi.OK
    assert np.array_equal(a.data, b.data)


def test_overlapping_node_ranges_are_rejected():
    w, h = 64, 64
    fills = random_fills(seed=12, n=3, w=w, h=h, side_lo=8, side_hi=40, seg_lo=3, seg_hi=6)
    nodes = np.concatenate([f[1] for f in fills])
    n0 = len(fills[0][1])
    # the third command draws the first one's nodes again
    fills3 = [fills[0], fills[1], (fills[2][0], fills[0][1], fills[2][2])]
    cmds, keep = _cmds(fills3, [0, n0, 0])
    s = _bg(w, h, 4)
    before = s.data.copy()
    with pytest.raises(Z2DError) as e:
        painter.fill_batch_arrays(s, nodes, cmds)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT and "share nodes" in str(e.value)
    assert np.array_equal(s.data, before)


def test_first_failing_command_decides_the_error():
    w, h = 128, 128
    fills = random_fills(seed=13, n=400, w=w, h=h, side_lo=4, side_hi=60, seg_lo=3, seg_hi=8)
    bad_px = Pattern.from_pixel(Pixel.rgba(200, 2, 3, 4))  # not premultiplied
    open_nodes = fills[150][1][:-2].copy()  # close_path and the move_to after it removed
    fills[150] = (fills[150][0], open_nodes, fills[150][2])
    fills[300] = (bad_px, fills[300][1], fills[300][2])
    nodes = np.concatenate([f[1] for f in fills])
    offs = np.concatenate([[0], np.cumsum([len(f[1]) for f in fills])[:-1]]).tolist()
    cmds, keep = _cmds(fills, offs)
    s = _bg(w, h, 5)
    before = s.data.copy()
    with pytest.raises(Z2DError) as e:
        painter.fill_batch_arrays(s, nodes, cmds)
    assert e.value.code == abi.ERR_PATH_NOT_CLOSED
    assert np.array_equal(s.data, before)
    fills[150] = random_fills(seed=13, n=400, w=w, h=h, side_lo=4, side_hi=60, seg_lo=3, seg_hi=8)[150]
    nodes = np.concatenate([f[1] for f in fills])
    offs = np.concatenate([[0], np.cumsum([len(f[1]) for f in fills])[:-1]]).tolist()
    cmds, keep = _cmds(fills, offs)
    with pytest.raises(Z2DError) as e:
        painter.fill_batch_arrays(s, nodes, cmds)
    assert e.value.code == abi.ERR_PIXEL_NOT_PREMULTIPLIED


def _square(x0=1.0):
    return [(abi.MOVE_TO, x0, 1, 0, 0, 0, 0), (abi.LINE_TO, 5, 1, 0, 0, 0, 0), (abi.LINE_TO, 5, 5, 0, 0, 0, 0),
            (abi.CLOSE_PATH, 0, 0, 0, 0, 0, 0)]


@pytest.mark.parametrize("case,code", [
    ("range_then_nan", abi.ERR_INVALID_ARGUMENT),   # coordinates are checked in order
    ("nan_then_range", abi.ERR_INVALID_STATE),
    ("inf", abi.ERR_INVALID_STATE),
    ("bad_tag", abi.ERR_INVALID_ARGUMENT),
    ("open_and_nan", abi.ERR_PATH_NOT_CLOSED),     # PathNotClosed comes first
])
def test_node_check_order(case, code):
    s = Surface.init("rgba", 8, 8)
    pat = Pattern.from_pixel(Pixel.rgba(1, 2, 3, 4))
    nodes = _square()
    if case == "range_then_nan":
        nodes[1] = (abi.LINE_TO, 2.0 ** 25, float("nan"), 0, 0, 0, 0)
    elif case == "nan_then_range":
        nodes[1] = (abi.LINE_TO, float("nan"), 2.0 ** 25, 0, 0, 0, 0)
    elif case == "inf":
        nodes[2] = (abi.LINE_TO, 5, float("-inf"), 0, 0, 0, 0)
    elif case == "bad_tag":
        nodes[2] = (9, 5, 5, 0, 0, 0, 0)
    else:
        nodes = nodes[:-1]
        nodes[1] = (abi.LINE_TO, float("nan"), 1, 0, 0, 0, 0)
    with pytest.raises(Z2DError) as e:
        painter.fill(s, pat, nodes, FillOptions())
    assert e.value.code == code
    assert not s.data.any()


def _draw_jobs_ops(rng_seed, n_jobs, per_job, w, h):
    from z2d_gb300.types import StrokeOptions
    fills = random_fills(seed=rng_seed, n=n_jobs * per_job, w=w, h=h, side_lo=4, side_hi=40, seg_lo=3, seg_hi=6)
    jobs = []
    for j in range(n_jobs):
        ops = []
        for k in range(per_job):
            pat, nodes, fo = fills[j * per_job + k]
            if k % 3 == 1:
                ops.append(("stroke", pat, nodes, StrokeOptions(line_width=2.0, dashes=(3.0, 2.0) if k % 2 else ())))
            else:
                ops.append(("fill", pat, nodes, fo))
        jobs.append(ops)
    return jobs


def test_draw_jobs_first_failing_entry_decides_the_error():
    """z2dgpu_draw_jobs prepares its (job, command) entries on host threads;
    the first failing entry in job order decides the error and no surface
    is drawn."""
    torch = pytest.importorskip("torch")
    w, h = 48, 40
    ops = _draw_jobs_ops(21, 12, 30, w, h)  # 360 entries: the threaded path
    bad_px = Pattern.from_pixel(Pixel.rgba(200, 2, 3, 4))
    k1 = ops[7][4]   # a stroke entry of job 7 (k % 3 == 1)
    ops[7][4] = (k1[0], bad_px, k1[2], k1[3])
    k2 = ops[9][3]   # a later fill entry with an open path
    ops[9][3] = (k2[0], k2[1], k2[2][:-2].copy(), k2[3])
    surfaces = [_bg(w, h, 30 + j).to_device("cuda") for j in range(12)]
    before = [s.to_host().data.copy() for s in surfaces]
    with pytest.raises(Z2DError) as e:
        painter.draw_jobs(list(zip(surfaces, ops)))
    assert e.value.code == abi.ERR_PIXEL_NOT_PREMULTIPLIED
    torch.cuda.synchronize()
    for s, b in zip(surfaces, before):
        assert np.array_equal(s.to_host().data, b)
    ops[7][4] = k1  # now the open path is the first failure
    with pytest.raises(Z2DError) as e:
        painter.draw_jobs(list(zip(surfaces, ops)))
    assert e.value.code == abi.ERR_PATH_NOT_CLOSED


def test_draw_jobs_threaded_matches_oracle(oracle):
    """A draw_jobs call large enough for the threaded preparation equals the
    commands drawn one by one by the oracle."""
    torch = pytest.importorskip("torch")
    import sys
    sys.path.insert(0, __import__("os").path.dirname(__file__))
    from backends import StrokeOracle
    w, h = 64, 48
    ops = _draw_jobs_ops(22, 10, 30, w, h)
    so = StrokeOracle(oracle)
    surfaces, refs = [], []
    for j in range(10):
        surfaces.append(_bg(w, h, 60 + j).to_device("cuda"))
        ref = _bg(w, h, 60 + j)
        for kind, pat, nodes, o in ops[j]:
            rc = oracle.fill(ref, pat, nodes, o) if kind == "fill" else so.stroke(ref, pat, nodes, o)
            assert rc == abi.OK
        refs.append(ref)
    painter.draw_jobs(list(zip(surfaces, ops)))
    torch.cuda.synchronize()
    for s, r in zip(surfaces, refs):
        assert np.array_equal(s.to_host().data, r.data)


def test_draw_jobs_many_nodes_matches_oracle(oracle):
    """A draw_jobs call of more than 2^20 nodes (200-segment paths, solid
    and dashed strokes among them) equals the oracle's drawing of each
    job's commands in order."""
    torch = pytest.importorskip("torch")
    import sys
    sys.path.insert(0, __import__("os").path.dirname(__file__))
    from backends import StrokeOracle
    from z2d_gb300.types import StrokeOptions
    w, h, n_jobs, per_job = 96, 80, 8, 660
    fills = random_fills(seed=23, n=n_jobs * per_job, w=w, h=h, side_lo=8, side_hi=80, seg_lo=200, seg_hi=200)
    assert sum(len(f[1]) for f in fills) > (1 << 20)
    so = StrokeOracle(oracle)
    ops, surfaces, refs = [], [], []
    for j in range(n_jobs):
        job = []
        for k in range(per_job):
            pat, nodes, fo = fills[j * per_job + k]
            if k % 40 == 7:
                job.append(("stroke", pat, nodes, StrokeOptions(line_width=1.5, dashes=(4.0, 3.0) if k % 80 == 7 else ())))
            else:
                job.append(("fill", pat, nodes, fo))
        ops.append(job)
        surfaces.append(_bg(w, h, 90 + j).to_device("cuda"))
        ref = _bg(w, h, 90 + j)
        for kind, pat, nodes, o in job:
            rc = oracle.fill(ref, pat, nodes, o) if kind == "fill" else so.stroke(ref, pat, nodes, o)
            assert rc == abi.OK
        refs.append(ref)
    painter.draw_jobs(list(zip(surfaces, ops)))
    torch.cuda.synchronize()
    for j, (s, r) in enumerate(zip(surfaces, refs)):
        assert np.array_equal(s.to_host().data, r.data), f"job {j}"
