"""Array packing for large batches.

painter.fill_batch / fill_jobs build one ctypes struct per command, which
costs microseconds each in Python.  For batches of 10^5+ fills the helpers
here write the C ABI structs (include/z2dgpu.h) directly into numpy arrays
whose layouts are taken from the ctypes declarations, so a whole batch is
packed with a few vectorised operations.  Pixel-pattern fills only.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import abi
from .native import Context, check, default_context


def _off(struct, field):
    return getattr(struct, field).offset


_PIX = _off(abi.z2d_pattern, "pixel")
PATTERN_DTYPE = np.dtype({
    "names": ["kind", "format", "r", "g", "b", "a", "dither_scale"],
    "formats": ["<i4", "<i4", "u1", "u1", "u1", "u1", "<i4"],
    "offsets": [_off(abi.z2d_pattern, "kind"), _PIX + _off(abi.z2d_pixel, "format"), _PIX + _off(abi.z2d_pixel, "r"),
                _PIX + _off(abi.z2d_pixel, "g"), _PIX + _off(abi.z2d_pixel, "b"), _PIX + _off(abi.z2d_pixel, "a"),
                _off(abi.z2d_pattern, "dither_scale")],
    "itemsize": C.sizeof(abi.z2d_pattern)})

_OPT = _off(abi.z2d_fill_cmd, "opts")
FILL_CMD_DTYPE = np.dtype({
    "names": ["pattern", "node_offset", "n_nodes", "anti_aliasing", "fill_rule", "op", "precision", "tolerance"],
    "formats": ["<u8", "<u8", "<u8", "<i4", "<i4", "<i4", "<i4", "<f8"],
    "offsets": [_off(abi.z2d_fill_cmd, "pattern"), _off(abi.z2d_fill_cmd, "node_offset"),
                _off(abi.z2d_fill_cmd, "n_nodes"), _OPT + _off(abi.z2d_fill_opts, "anti_aliasing"),
                _OPT + _off(abi.z2d_fill_opts, "fill_rule"), _OPT + _off(abi.z2d_fill_opts, "op"),
                _OPT + _off(abi.z2d_fill_opts, "precision"), _OPT + _off(abi.z2d_fill_opts, "tolerance")],
    "itemsize": C.sizeof(abi.z2d_fill_cmd)})

_SFC = _off(abi.z2d_job, "surface")
JOB_DTYPE = np.dtype({
    "names": ["format", "width", "height", "location", "data", "cmd_offset", "n_cmds"],
    "formats": ["<i4", "<i4", "<i4", "<i4", "<u8", "<u8", "<u8"],
    "offsets": [_SFC + _off(abi.z2d_surface, f) for f in ("format", "width", "height", "location", "data")] +
               [_off(abi.z2d_job, "cmd_offset"), _off(abi.z2d_job, "n_cmds")],
    "itemsize": C.sizeof(abi.z2d_job)})


class PackedBatch:
    """C ABI arrays of a pixel-pattern batch: nodes, patterns, commands and
    (for multi-surface batches) jobs.  The command array points into the
    pattern array, so both live as long as this object."""

    def __init__(self, nodes: np.ndarray, node_offsets: np.ndarray, node_counts: np.ndarray, pixels: np.ndarray,
                 fill_rules: np.ndarray, anti_aliasing: int = abi.AA_DEFAULT, op: int = abi.OP["src_over"],
                 precision: int = abi.PRECISION_INTEGER, tolerance: float = 0.1):
        n = len(node_offsets)
        self.nodes = np.ascontiguousarray(nodes)
        self.patterns = np.zeros(n, PATTERN_DTYPE)
        self.patterns["kind"] = abi.PATTERN_PIXEL
        self.patterns["format"] = abi.FORMAT_RGBA
        self.patterns["dither_scale"] = 8  # Pattern's default; unused by pixel sources
        for i, ch in enumerate("rgba"):
            self.patterns[ch] = pixels[:, i]
        self.cmds = np.zeros(n, FILL_CMD_DTYPE)
        self.cmds["pattern"] = self.patterns.ctypes.data + np.arange(n, dtype=np.uint64) * PATTERN_DTYPE.itemsize
        self.cmds["node_offset"] = node_offsets
        self.cmds["n_nodes"] = node_counts
        self.cmds["anti_aliasing"] = anti_aliasing
        self.cmds["fill_rule"] = fill_rules
        self.cmds["op"] = op
        self.cmds["precision"] = precision
        self.cmds["tolerance"] = tolerance
        self.jobs: Optional[np.ndarray] = None

    def set_jobs(self, surfaces: Sequence, cmd_offsets: Sequence[int], cmd_counts: Sequence[int]) -> None:
        """One job per device surface (z2d_gb300.surface.Surface), drawing
        commands [cmd_offsets[j], cmd_offsets[j] + cmd_counts[j])."""
        self.jobs = np.zeros(len(surfaces), JOB_DTYPE)
        for j, s in enumerate(surfaces):
            a = s.to_abi()
            self.jobs[j] = (a.format, a.width, a.height, a.location, a.data or 0, cmd_offsets[j], cmd_counts[j])

    def fill_jobs(self, ctx: Optional[Context] = None) -> None:
        ctx = ctx or default_context()
        check(ctx.lib.z2dgpu_fill_jobs(ctx.handle, self.jobs.ctypes.data_as(C.POINTER(abi.z2d_job)), len(self.jobs),
                                       self.nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(self.nodes),
                                       self.cmds.ctypes.data_as(C.POINTER(abi.z2d_fill_cmd)), len(self.cmds)))

    def fill_batch(self, surface, first: int = 0, count: Optional[int] = None, ctx: Optional[Context] = None) -> None:
        """Commands [first, first + count) on one surface (z2dgpu_fill_batch)."""
        ctx = ctx or default_context()
        count = len(self.cmds) - first if count is None else count
        if count <= 0:
            return
        s = surface.to_abi()
        cmds = self.cmds[first:first + count].copy()
        # pass only the node range these commands use
        lo = int(cmds["node_offset"].min())
        hi = int((cmds["node_offset"] + cmds["n_nodes"]).max())
        cmds["node_offset"] -= lo
        nodes = self.nodes[lo:hi]
        check(ctx.lib.z2dgpu_fill_batch(ctx.handle, C.byref(s), nodes.ctypes.data_as(C.POINTER(abi.z2d_node)),
                                        len(nodes), cmds.ctypes.data_as(C.POINTER(abi.z2d_fill_cmd)), count))


_FILL = _off(abi.z2d_draw_cmd, "fill")
_STROKE = _off(abi.z2d_draw_cmd, "stroke")


def _so(field):
    return _STROKE + _off(abi.z2d_stroke_opts, field)


# Every byte of the C struct is a named field: numpy copies of structured
# arrays transfer fields only, so unnamed gaps would come out undefined.
DRAW_CMD_DTYPE = np.dtype({
    "names": ["kind", "_pad", "pattern", "node_offset", "n_nodes", "f_aa", "f_rule", "f_op", "f_precision",
              "f_tolerance", "s_aa", "s_join", "s_cap", "s_op", "s_precision", "s_hairline", "s_line_width",
              "s_miter_limit", "s_tolerance", "s_dash_offset", "s_tf", "s_dashes", "s_n_dashes"],
    "formats": ["<i4", "<i4", "<u8", "<u8", "<u8", "<i4", "<i4", "<i4", "<i4", "<f8",
                "<i4", "<i4", "<i4", "<i4", "<i4", "<i4", "<f8", "<f8", "<f8", "<f8", ("<f8", (6,)), "<u8", "<u8"],
    "offsets": [_off(abi.z2d_draw_cmd, "kind"), _off(abi.z2d_draw_cmd, "_pad"), _off(abi.z2d_draw_cmd, "pattern"),
                _off(abi.z2d_draw_cmd, "node_offset"), _off(abi.z2d_draw_cmd, "n_nodes"),
                _FILL + _off(abi.z2d_fill_opts, "anti_aliasing"), _FILL + _off(abi.z2d_fill_opts, "fill_rule"),
                _FILL + _off(abi.z2d_fill_opts, "op"), _FILL + _off(abi.z2d_fill_opts, "precision"),
                _FILL + _off(abi.z2d_fill_opts, "tolerance"),
                _so("anti_aliasing"), _so("line_join"), _so("line_cap"), _so("op"), _so("precision"),
                _so("hairline"), _so("line_width"), _so("miter_limit"), _so("tolerance"), _so("dash_offset"), _so("transformation"),
                _so("dashes"), _so("n_dashes")],
    "itemsize": C.sizeof(abi.z2d_draw_cmd)})


class PackedDrawBatch(PackedBatch):
    """PackedBatch whose commands may be strokes (z2dgpu_draw_jobs): where
    stroke[i] is set, command i strokes its nodes with width widths[i],
    join joins[i], cap caps[i] and the dash array dashes[i] (empty: solid)."""

    def __init__(self, nodes, node_offsets, node_counts, pixels, fill_rules, stroke, widths, joins, caps, dashes,
                 anti_aliasing: int = abi.AA_DEFAULT):
        super().__init__(nodes, node_offsets, node_counts, pixels, fill_rules, anti_aliasing)
        n = len(node_offsets)
        flat = [float(v) for d in dashes for v in d]
        self.dash_values = np.array(flat if flat else [0.0], np.float64)
        dash_off = np.zeros(n, np.int64)
        if n:
            np.cumsum([len(d) for d in dashes][:-1], out=dash_off[1:])
        d = np.zeros(n, DRAW_CMD_DTYPE)
        d["kind"] = np.where(stroke, abi.DRAW_STROKE, abi.DRAW_FILL)
        d["pattern"] = self.cmds["pattern"]
        d["node_offset"] = node_offsets
        d["n_nodes"] = node_counts
        d["f_aa"] = anti_aliasing
        d["f_rule"] = fill_rules
        d["f_op"] = abi.OP["src_over"]
        d["f_precision"] = abi.PRECISION_INTEGER
        d["f_tolerance"] = 0.1
        d["s_aa"] = anti_aliasing
        d["s_join"] = joins
        d["s_cap"] = caps
        d["s_op"] = abi.OP["src_over"]
        d["s_precision"] = abi.PRECISION_INTEGER
        d["s_line_width"] = widths
        d["s_miter_limit"] = 10.0
        d["s_tolerance"] = 0.1
        d["s_tf"] = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
        nd = np.array([len(x) for x in dashes], np.uint64)
        d["s_n_dashes"] = nd
        d["s_dashes"] = np.where(nd > 0, self.dash_values.ctypes.data + dash_off.astype(np.uint64) * 8, 0)
        self.draw_cmds = d

    def draw_jobs(self, ctx: Optional[Context] = None) -> None:
        ctx = ctx or default_context()
        check(ctx.lib.z2dgpu_draw_jobs(ctx.handle, self.jobs.ctypes.data_as(C.POINTER(abi.z2d_job)), len(self.jobs),
                                       self.nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(self.nodes),
                                       self.draw_cmds.ctypes.data_as(C.POINTER(abi.z2d_draw_cmd)),
                                       len(self.draw_cmds)))

    def draw_job(self, j: int, ctx: Optional[Context] = None) -> None:
        """Job j alone (z2dgpu_draw_jobs with one job and only its nodes)."""
        ctx = ctx or default_context()
        jb = self.jobs[j:j + 1].copy()
        c0, n = int(jb["cmd_offset"][0]), int(jb["n_cmds"][0])
        if n == 0:
            return
        cmds = self.draw_cmds[c0:c0 + n].copy()
        lo = int(cmds["node_offset"].min())
        hi = int((cmds["node_offset"] + cmds["n_nodes"]).max())
        cmds["node_offset"] -= lo
        jb["cmd_offset"] = 0
        nodes = self.nodes[lo:hi]
        check(ctx.lib.z2dgpu_draw_jobs(ctx.handle, jb.ctypes.data_as(C.POINTER(abi.z2d_job)), 1,
                                       nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(nodes),
                                       cmds.ctypes.data_as(C.POINTER(abi.z2d_draw_cmd)), n))
