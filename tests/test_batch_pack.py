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


def test_draw_cmd_dtype_matches_ctypes():
    from z2d_gb300.batch import DRAW_CMD_DTYPE, PackedDrawBatch
    from z2d_gb300.types import StrokeOptions
    assert DRAW_CMD_DTYPE.itemsize == C.sizeof(abi.z2d_draw_cmd)
    job = batched_jobs(seed=8, n_jobs=1, side_lo=64, side_hi=64, paths_lo=6, paths_hi=6)[0]
    w, h, nodes, off, cnt, px, rules = job
    stroke = np.array([False, True, False, True, True, False])
    widths = np.array([2.0, 3.5, 2.0, 0.75, 12.0, 2.0])
    joins = np.array([0, 1, 0, 2, 0, 0])
    caps = np.array([0, 2, 0, 1, 0, 0])
    dashes = [(), (4.0, 2.0), (), (), (1.0, 3.0, 5.0), ()]
    pb = PackedDrawBatch(nodes, off, cnt, px, rules, stroke, widths, joins, caps, dashes)
    keep = []
    for i in range(6):
        cmd = abi.z2d_draw_cmd()
        cmd.kind = abi.DRAW_STROKE if stroke[i] else abi.DRAW_FILL
        cmd.node_offset = int(off[i])
        cmd.n_nodes = int(cnt[i])
        cmd.fill = FillOptions(fill_rule="even_odd" if rules[i] == abi.FILL_EVEN_ODD else "non_zero").to_abi()
        so = StrokeOptions(line_width=float(widths[i]), line_join=("miter", "round", "bevel")[joins[i]],
                           line_cap=("butt", "round", "square")[caps[i]], dashes=dashes[i])
        cmd.stroke = so.to_abi(keep)
        got = bytearray(pb.draw_cmds[i].tobytes())
        exp = bytearray(_bytes(cmd))
        for field in ("pattern",):  # pointers differ by construction
            o = getattr(abi.z2d_draw_cmd, field).offset
            got[o:o + 8] = exp[o:o + 8] = bytes(8)
        o = abi.z2d_draw_cmd.stroke.offset + abi.z2d_stroke_opts.dashes.offset
        assert int.from_bytes(got[o:o + 8], "little") != 0 or not dashes[i]
        got[o:o + 8] = exp[o:o + 8] = bytes(8)
        assert bytes(got) == bytes(exp), i


def test_packed_dtypes_have_no_gaps():
    """numpy copies structured arrays field by field: every byte of the C
    structs that are copied (commands, jobs) must belong to a field."""
    from z2d_gb300.batch import DRAW_CMD_DTYPE
    for dt in (DRAW_CMD_DTYPE, FILL_CMD_DTYPE, JOB_DTYPE):
        assert sum(dt.fields[n][0].itemsize for n in dt.names) == dt.itemsize
    from z2d_gb300.batch import PackedDrawBatch
    job = batched_jobs(seed=9, n_jobs=1, side_lo=32, side_hi=32, paths_lo=4, paths_hi=4)[0]
    w, h, nodes, off, cnt, px, rules = job
    pb = PackedDrawBatch(nodes, off, cnt, px, rules, np.ones(4, bool), np.full(4, 3.0), np.zeros(4, int),
                         np.zeros(4, int), [()] * 4)
    assert pb.draw_cmds[1:3].copy().tobytes() == pb.draw_cmds[1:3].tobytes()
