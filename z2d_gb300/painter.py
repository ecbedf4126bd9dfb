"""painter.fill with z2d's signature, running on the GPU (libz2dgpu.so).

Mirrors src/painter.zig:66-143: the same options, defaults and errors
(raised as native.Z2DError with z2d's error names).  fill_batch is the
batched form: N fills on one surface in call order, one device pass.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from . import abi
from .native import Context, check, default_context
from .types import NODE_DTYPE, FillOptions, Pattern, nodes_to_abi


def fill(surface, pattern: Pattern, nodes, opts: FillOptions = FillOptions(), ctx: Optional[Context] = None) -> None:
    """Fills the path `nodes` onto `surface` with `pattern`."""
    ctx = ctx or default_context()
    keep: list = []
    s = surface.to_abi()
    p = pattern.to_abi(keep)
    arr = nodes_to_abi(nodes)
    check(ctx.lib.z2dgpu_fill(ctx.handle, C.byref(s), C.byref(p), arr, len(nodes), C.byref(opts.to_abi())))


def fill_batch(surface, fills: Sequence[Tuple[Pattern, object, FillOptions]], ctx: Optional[Context] = None) -> None:
    """Equivalent to fill() for each (pattern, nodes, opts) in order."""
    ctx = ctx or default_context()
    keep: list = []
    node_arrays = []
    cmds = (abi.z2d_fill_cmd * max(1, len(fills)))()
    off = 0
    for i, (pat, nodes, opts) in enumerate(fills):
        arr = nodes if isinstance(nodes, np.ndarray) and nodes.dtype == NODE_DTYPE else None
        if arr is None:
            from .path import nodes_array
            arr = nodes_array(nodes)
        node_arrays.append(arr)
        p = pat.to_abi(keep)
        cmds[i].pattern = C.pointer(p)
        cmds[i].node_offset = off
        cmds[i].n_nodes = len(arr)
        cmds[i].opts = opts.to_abi()
        off += len(arr)
    all_nodes = np.concatenate(node_arrays) if node_arrays else np.zeros(0, NODE_DTYPE)
    all_nodes = np.ascontiguousarray(all_nodes)
    s = surface.to_abi()
    check(ctx.lib.z2dgpu_fill_batch(ctx.handle, C.byref(s),
                                    all_nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(all_nodes),
                                    cmds, len(fills)))


def fill_batch_arrays(surface, nodes: np.ndarray, cmds, ctx: Optional[Context] = None) -> None:
    """Low-level batch entry: a NODE_DTYPE array and a ctypes z2d_fill_cmd
    array that indexes into it (no per-call marshalling)."""
    ctx = ctx or default_context()
    s = surface.to_abi()
    check(ctx.lib.z2dgpu_fill_batch(ctx.handle, C.byref(s), nodes.ctypes.data_as(C.POINTER(abi.z2d_node)),
                                    len(nodes), cmds, len(cmds)))


def fill_jobs(jobs: Sequence[Tuple[object, Sequence[Tuple[Pattern, object, FillOptions]]]],
              ctx: Optional[Context] = None) -> None:
    """Many surfaces in one device pass: for each (surface, fills) job, the
    equivalent of fill() for each (pattern, nodes, opts) in order on that
    surface.  Surfaces must be device-resident (Surface.to_device) and
    distinct."""
    ctx = ctx or default_context()
    keep: list = []
    node_arrays = []
    n_cmds = sum(len(f) for _, f in jobs)
    cmds = (abi.z2d_fill_cmd * max(1, n_cmds))()
    jarr = (abi.z2d_job * max(1, len(jobs)))()
    off = 0
    ci = 0
    for j, (surface, fills) in enumerate(jobs):
        jarr[j].surface = surface.to_abi()
        jarr[j].cmd_offset = ci
        jarr[j].n_cmds = len(fills)
        for pat, nodes, opts in fills:
            arr = nodes if isinstance(nodes, np.ndarray) and nodes.dtype == NODE_DTYPE else None
            if arr is None:
                from .path import nodes_array
                arr = nodes_array(nodes)
            node_arrays.append(arr)
            p = pat.to_abi(keep)
            cmds[ci].pattern = C.pointer(p)
            cmds[ci].node_offset = off
            cmds[ci].n_nodes = len(arr)
            cmds[ci].opts = opts.to_abi()
            off += len(arr)
            ci += 1
    all_nodes = np.ascontiguousarray(np.concatenate(node_arrays) if node_arrays else np.zeros(0, NODE_DTYPE))
    check(ctx.lib.z2dgpu_fill_jobs(ctx.handle, jarr, len(jobs), all_nodes.ctypes.data_as(C.POINTER(abi.z2d_node)),
                                   len(all_nodes), cmds, n_cmds))


def fill_jobs_arrays(jarr, nodes: np.ndarray, cmds, ctx: Optional[Context] = None) -> None:
    """Low-level multi-surface entry: ctypes z2d_job and z2d_fill_cmd arrays
    and the NODE_DTYPE array they index (no per-call marshalling)."""
    ctx = ctx or default_context()
    check(ctx.lib.z2dgpu_fill_jobs(ctx.handle, jarr, len(jarr), nodes.ctypes.data_as(C.POINTER(abi.z2d_node)),
                                   len(nodes), cmds, len(cmds)))


def stroke(surface, pattern: Pattern, nodes, opts: Optional["StrokeOptions"] = None,
           ctx: Optional[Context] = None) -> None:
    """painter.stroke (src/painter.zig:214-344): the stroke polygon is built
    on the host like z2d's stroke plotter, then filled on the GPU."""
    from .types import StrokeOptions
    ctx = ctx or default_context()
    opts = opts or StrokeOptions()
    keep: list = []
    arr = nodes_to_abi(nodes)
    s = surface.to_abi()
    p = pattern.to_abi(keep)
    o = opts.to_abi(keep)
    check(ctx.lib.z2dgpu_stroke(ctx.handle, C.byref(s), C.byref(p), arr, len(arr), C.byref(o)))


def stroke_contours(nodes, opts: Optional["StrokeOptions"] = None, surface_format="rgba"):
    """The stroke polygon painter.stroke rasterises on a surface of
    `surface_format`: (list of (n, 2) arrays of already-scaled points, one
    per closed contour, and the rasteriser scale).  Host only."""
    from .native import load
    from .types import StrokeOptions, _fmt
    lib = load()
    opts = opts or StrokeOptions()
    keep: list = []
    arr = nodes_to_abi(nodes)
    o = opts.to_abi(keep)
    npts, nc, sc = C.c_uint64(), C.c_uint64(), C.c_double()
    fmt = _fmt(surface_format)
    check(lib.z2dgpu_stroke_contours(arr, len(arr), C.byref(o), fmt, None, 0, C.byref(npts), None, 0, C.byref(nc),
                                     C.byref(sc)))
    pts = np.zeros(max(1, npts.value) * 2, np.float64)
    ends = np.zeros(max(1, nc.value), np.uint64)
    check(lib.z2dgpu_stroke_contours(arr, len(arr), C.byref(o), fmt, pts.ctypes.data_as(C.POINTER(C.c_double)),
                                     npts.value, C.byref(npts), ends.ctypes.data_as(C.POINTER(C.c_uint64)), nc.value,
                                     C.byref(nc), C.byref(sc)))
    out, start = [], 0
    for e in ends[:nc.value]:
        out.append(pts[2 * start:2 * int(e)].reshape(-1, 2).copy())
        start = int(e)
    return out, sc.value


def draw_jobs(jobs, ctx: Optional[Context] = None) -> None:
    """Fills and strokes over many surfaces in one pass: jobs is a sequence
    of (surface, ops) with ops a sequence of ("fill", pattern, nodes,
    FillOptions) or ("stroke", pattern, nodes, StrokeOptions), drawn in
    order on their device-resident surface."""
    ctx = ctx or default_context()
    keep: list = []
    node_arrays = []
    n_cmds = sum(len(o) for _, o in jobs)
    cmds = (abi.z2d_draw_cmd * max(1, n_cmds))()
    jarr = (abi.z2d_job * max(1, len(jobs)))()
    off = ci = 0
    for j, (surface, ops) in enumerate(jobs):
        jarr[j].surface = surface.to_abi()
        jarr[j].cmd_offset = ci
        jarr[j].n_cmds = len(ops)
        for kind, pat, nodes, opts in ops:
            arr = nodes if isinstance(nodes, np.ndarray) and nodes.dtype == NODE_DTYPE else None
            if arr is None:
                from .path import nodes_array
                arr = nodes_array(nodes)
            node_arrays.append(arr)
            p = pat.to_abi(keep)
            cmds[ci].pattern = C.pointer(p)
            cmds[ci].node_offset = off
            cmds[ci].n_nodes = len(arr)
            if kind == "fill":
                cmds[ci].kind = abi.DRAW_FILL
                cmds[ci].fill = opts.to_abi()
            else:
                cmds[ci].kind = abi.DRAW_STROKE
                cmds[ci].stroke = opts.to_abi(keep)
            off += len(arr)
            ci += 1
    all_nodes = np.ascontiguousarray(np.concatenate(node_arrays) if node_arrays else np.zeros(0, NODE_DTYPE))
    check(ctx.lib.z2dgpu_draw_jobs(ctx.handle, jarr, len(jobs), all_nodes.ctypes.data_as(C.POINTER(abi.z2d_node)),
                                   len(all_nodes), cmds, n_cmds))
