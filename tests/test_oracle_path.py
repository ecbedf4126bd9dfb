"""The oracle's Path builder (oracle/z2d_path.cpp) pinned to z2d.

* Known answers of z2d's own Path tests (src/Path.zig:574-915): clamping to
  the i24 range, the rel* helpers (also under a translation) and their
  NoCurrentPoint errors.
* The restated Zig f64 sin / cos / tan against the host libm: both are
  faithful (< 1 ulp), so they may differ by one ulp but never more.
* Random programs against the package's Python Path mirror (z2d_gb300.path),
  which follows the same Zig code: identical nodes without arcs; with arcs,
  the same node count and coordinates within the trigonometry's last ulp
  (the mirror uses the host libm's sin / cos / tan, the oracle Zig's).
"""
import math

import numpy as np
import pytest

from z2d_gb300 import abi
from z2d_gb300.path import Path
from z2d_gb300.path_program import PathProgram

I24_MIN, I24_MAX = -(1 << 23), (1 << 23) - 1


def _nodes(oracle, prog):
    nodes, status = oracle.build_paths([prog])
    return [(int(n["tag"]), *map(float, n["p"])) for n in nodes[0]], status[0]


def _node(tag, *p):
    return (tag, *(list(p) + [0.0] * (6 - len(p))))


def test_clamped_kats(oracle):
    """Path.zig:574-687: moveTo / lineTo / curveTo clamp to the i24 range."""
    nodes, st = _nodes(oracle, PathProgram().move_to(I24_MIN - 1, I24_MAX + 1))
    assert st == 0 and nodes == [_node(abi.MOVE_TO, I24_MIN, I24_MAX)]
    nodes, st = _nodes(oracle, PathProgram().move_to(1, 1).line_to(I24_MIN - 1, I24_MAX + 1))
    assert nodes[1] == _node(abi.LINE_TO, I24_MIN, I24_MAX)
    p = PathProgram().move_to(1, 1).curve_to(I24_MIN - 1, I24_MAX + 1, 3, 4, 5, 6)
    p.curve_to(1, 2, I24_MIN - 1, I24_MAX + 1, 5, 6).curve_to(1, 2, 3, 4, I24_MIN - 1, I24_MAX + 1)
    nodes, st = _nodes(oracle, p)
    assert nodes[1:] == [_node(abi.CURVE_TO, I24_MIN, I24_MAX, 3, 4, 5, 6),
                         _node(abi.CURVE_TO, 1, 2, I24_MIN, I24_MAX, 5, 6),
                         _node(abi.CURVE_TO, 1, 2, 3, 4, I24_MIN, I24_MAX)]


def test_relative_kats(oracle):
    """Path.zig:763-875: rel* from the current point, NoCurrentPoint without one."""
    nodes, _ = _nodes(oracle, PathProgram().move_to(1, 1).rel_move_to(-10, -10))
    assert nodes == [_node(abi.MOVE_TO, 1, 1), _node(abi.MOVE_TO, -9, -9)]
    nodes, _ = _nodes(oracle, PathProgram().move_to(1, 1).rel_line_to(1, 1))
    assert nodes[1] == _node(abi.LINE_TO, 2, 2)
    nodes, _ = _nodes(oracle, PathProgram().move_to(1, 1).rel_curve_to(-10, -10, -11, -11, -12, -12))
    assert nodes[1] == _node(abi.CURVE_TO, -9, -9, -10, -10, -11, -11)
    for prog in (PathProgram().rel_move_to(1, 1), PathProgram().rel_line_to(1, 1),
                 PathProgram().rel_curve_to(1, 1, 2, 2, 3, 3)):
        nodes, st = _nodes(oracle, prog)
        assert nodes == [] and st == abi.ERR_INVALID_STATE


def test_relative_with_transformation_kat(oracle):
    """Path.zig:877-915: the helpers under translate(100, 200)."""
    t = (1.0, 0.0, 0.0, 1.0, 100.0, 200.0)
    nodes, _ = _nodes(oracle, PathProgram(t).move_to(0, 0).rel_move_to(-10, -20))
    assert nodes == [_node(abi.MOVE_TO, 100, 200), _node(abi.MOVE_TO, 90, 180)]
    nodes, _ = _nodes(oracle, PathProgram(t).move_to(0, 0).rel_move_to(-10, -20).reset().move_to(0, 0)
                      .rel_line_to(-10, -20))
    assert nodes[1] == _node(abi.LINE_TO, 90, 180)
    nodes, _ = _nodes(oracle, PathProgram(t).move_to(0, 0).rel_curve_to(-10, -20, 30, 40, -50, -60))
    assert nodes[1] == _node(abi.CURVE_TO, 90, 180, 130, 240, 50, 140)


def _ulps(a, b):
    if a == b:
        return 0
    ia = np.array([a]).view(np.int64)[0]
    ib = np.array([b]).view(np.int64)[0]
    return abs(int(ia) - int(ib))


@pytest.mark.parametrize("which", ["sin", "cos", "tan"])
def test_zig_trig_faithful(oracle, which):
    rng = np.random.default_rng({"sin": 1, "cos": 2, "tan": 3}[which])
    xs = np.concatenate([rng.uniform(-7, 7, 4000), rng.uniform(-1e5, 1e5, 2000), rng.uniform(-1e-6, 1e-6, 200),
                         np.array([0.0, math.pi / 4, math.pi / 2, math.pi, 3 * math.pi / 2, 2 * math.pi,
                                   1.5707963267948966, 4.71238898038469, 1e6, -1e6])])
    ref = getattr(math, which)
    worst = max(_ulps(oracle.zig_trig(which, float(x)), ref(float(x))) for x in xs)
    assert worst <= 1, f"{which}: {worst} ulps from the host libm"
    assert oracle.zig_trig(which, 1e7) is None  # beyond the medium reduction range


def _random_program(rng, arcs: bool) -> tuple:
    t = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    if rng.random() < 0.6:
        a = rng.uniform(-math.pi, math.pi)
        sx, sy = rng.uniform(0.25, 4, 2)
        c, s = math.cos(a), math.sin(a)
        t = (c * sx, -s * sy, s * sx, c * sy, rng.uniform(-300, 300), rng.uniform(-300, 300))
    prog, mirror = PathProgram(t, tolerance=float(rng.choice([0.1, 0.01, 0.5]))), Path(t, 0.1)
    mirror.tolerance = prog.tolerance
    for _ in range(int(rng.integers(1, 30))):
        r = rng.random()
        x, y = rng.uniform(-500, 500, 2)
        if r < 0.15:
            prog.move_to(x, y), mirror.move_to(x, y)
        elif r < 0.45:
            prog.line_to(x, y), mirror.line_to(x, y)
        elif r < 0.6 and mirror.current is not None:
            c = rng.uniform(-500, 500, 4)
            prog.curve_to(*c, x, y), mirror.curve_to(*c, x, y)
        elif r < 0.7 and mirror.current is not None:
            prog.rel_line_to(x / 10, y / 10), mirror.rel_line_to(x / 10, y / 10)
        elif r < 0.8:
            prog.close(), mirror.close()
        elif arcs:
            rad = rng.uniform(1, 200)
            a1, a2 = rng.uniform(-10, 10, 2)
            if rng.random() < 0.5:
                prog.arc(x, y, rad, a1, a2), mirror.arc(x, y, rad, a1, a2)
            else:
                prog.arc_negative(x, y, rad, a1, a2), mirror.arc_negative(x, y, rad, a1, a2)
    return prog, mirror


def test_programs_match_mirror_without_arcs(oracle):
    rng = np.random.default_rng(11)
    pairs = [_random_program(rng, arcs=False) for _ in range(300)]
    built, status = oracle.build_paths([p for p, _ in pairs])
    for k, ((_, mirror), nodes) in enumerate(zip(pairs, built)):
        want = mirror.to_array()
        assert status[k] == 0
        assert len(nodes) == len(want) and np.array_equal(nodes["tag"], want["tag"]), k
        assert np.array_equal(nodes["p"], want["p"]), k


def test_programs_close_to_mirror_with_arcs(oracle):
    rng = np.random.default_rng(12)
    pairs = [_random_program(rng, arcs=True) for _ in range(200)]
    built, status = oracle.build_paths([p for p, _ in pairs])
    for k, ((_, mirror), nodes) in enumerate(zip(pairs, built)):
        want = mirror.to_array()
        assert status[k] == 0
        assert len(nodes) == len(want) and np.array_equal(nodes["tag"], want["tag"]), k
        np.testing.assert_allclose(nodes["p"], want["p"], rtol=1e-12, atol=1e-9, err_msg=str(k))


def test_glyph_outline_kat(oracle):
    """Glyph.zig:876-967: glyph 56 ('a') of the test font has advance 1150
    and its outline is closed and holds curves (the fixture is decoded from
    the font by tests/golden/extract_glyphs.py)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "glyphs_inter_regular.json")) as f:
        fx = json.load(f)
    g = fx["glyphs"][0]
    assert g["index"] == 56 and g["advance"] == 1150 and fx["units_per_em"] == 2048
    nodes, st = _nodes(oracle, PathProgram().glyph([tuple(q) for q in g["points"]], g["ends"], 2048))
    assert st == 0
    tags = [n[0] for n in nodes]
    assert abi.CURVE_TO in tags
    # PathNode.isClosedNodeSet: every subpath that draws ends in close_path
    drawing = False
    for t in tags:
        if t == abi.MOVE_TO:
            assert not drawing
        elif t == abi.CLOSE_PATH:
            drawing = False
        else:
            drawing = True
    assert not drawing
    # y flipped into device space: font units up, device y down
    ys = [n[2] for n in nodes if n[0] in (abi.MOVE_TO, abi.LINE_TO)]
    assert min(ys) >= 2048 - max(p[1] for p in g["points"]) - 1e-9
