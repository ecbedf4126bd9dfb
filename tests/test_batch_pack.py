"""The numpy batch packer writes the same bytes as the ctypes structs."""
import ctypes as C

import numpy as np

from z2d_gb300 import abi
from z2d_gb300.batch import FILL_CMD_DTYPE, JOB_DTYPE, PATTERN_DTYPE, PackedBatch
from z2d_gb300.types import FillOptions, Pattern, Pixel
from z2d_gb300.workloads import batched_jobs, job_fills


def _bytes(struct):
    return bytes(memoryview(struct).cast("B"))


def test_dtype_sizes_match_ctypes():
    assert PATTERN_DTYPE.itemsize == C.sizeof(abi.z2d_pattern)
    assert FILL_CMD_DTYPE.itemsize == C.sizeof(abi.z2d_fill_cmd)
    assert JOB_DTYPE.itemsize == C.sizeof(abi.z2d_job)


def test_packed_commands_match_ctypes():
    job = batched_jobs(seed=5, n_jobs=1, side_lo=64, side_hi=64, paths_lo=20, paths_hi=20)[0]
    w, h, nodes, off, cnt, px, rules = job
    pb = PackedBatch(nodes, off, cnt, px, rules)
    keep = []
    for i, (pat, nds, opts) in enumerate(job_fills(job)):
        p = pat.to_abi(keep)
        assert _bytes(p) == pb.patterns[i].tobytes()
        cmd = abi.z2d_fill_cmd()
        cmd.node_offset = int(off[i])
        cmd.n_nodes = int(cnt[i])
        cmd.opts = opts.to_abi()
        got = bytearray(pb.cmds[i].tobytes())
        ptr = int(pb.cmds[i]["pattern"])
        assert ptr == pb.patterns.ctypes.data + i * PATTERN_DTYPE.itemsize
        got[:8] = bytes(8)  # the pattern pointer differs by construction
        assert bytes(got) == _bytes(cmd)
        assert np.array_equal(nodes[off[i]:off[i] + cnt[i]], nds)


def test_generated_paths_are_closed_subpaths():
    job = batched_jobs(seed=6, n_jobs=1, side_lo=100, side_hi=100, paths_lo=50, paths_hi=50)[0]
    w, h, nodes, off, cnt, px, rules = job
    for i in range(len(off)):
        p = nodes[off[i]:off[i] + cnt[i]]
        assert p["tag"][0] == abi.MOVE_TO and p["tag"][-2] == abi.CLOSE_PATH and p["tag"][-1] == abi.MOVE_TO
        assert np.array_equal(p["p"][-1][:2], p["p"][0][:2])
        assert set(p["tag"][1:-2]) <= {abi.LINE_TO, abi.CURVE_TO}
        assert (px[i, :3] <= px[i, 3]).all() and px[i, 3] >= 32
