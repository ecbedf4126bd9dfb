"""Continuous batching in front of the multi-surface fill pass
(z2dgpu_server_*).

    srv = Server(max_batch_jobs=256, max_wait_us=200, lanes=2, pool_bytes=1 << 30)
    t = srv.submit(surface, [(pattern, nodes, opts), ...])    # caller's device surface
    out = np.empty(w * h * 4, np.uint8)
    t2 = srv.submit_new("rgba", w, h, fills, init=None, out=out)  # a pool surface, read back into `out`
    latency_us = srv.wait(t)                                  # raises Z2DError on failure
    srv.close()

Several lanes draw batches concurrently; requests on a pool surface are
admitted once the pool has room for it.  Caller-owned surfaces must be
device-resident (Surface.to_device) and stay alive until their requests
complete; requests on one surface are drawn in submission order.  There is
no counterpart in z2d: it is the serving loop around painter.fill.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from . import abi
from .native import Z2DError, check, load
from .types import NODE_DTYPE, FillOptions, Pattern


class Server:
    def __init__(self, device: int = 0, max_batch_jobs: int = 256, max_wait_us: int = 200, lanes: int = 2,
                 pool_bytes: int = 0):
        self.lib = load()
        self.handle = C.c_void_p()
        self._outs = {}  # ticket -> output buffer kept alive until wait()
        opts = abi.z2dgpu_server_opts(max_batch_jobs=max_batch_jobs, max_wait_us=max_wait_us, lanes=lanes,
                                      pool_bytes=pool_bytes)
        check(self.lib.z2dgpu_server_create2(C.byref(self.handle), device, C.byref(opts)))

    @staticmethod
    def _pack(fills):
        keep: list = []
        arrays = []
        cmds = (abi.z2d_fill_cmd * max(1, len(fills)))()
        off = 0
        for i, (pat, nodes, opts) in enumerate(fills):
            arr = nodes if isinstance(nodes, np.ndarray) and nodes.dtype == NODE_DTYPE else None
            if arr is None:
                from .path import nodes_array
                arr = nodes_array(nodes)
            arrays.append(arr)
            p = pat.to_abi(keep)
            cmds[i].pattern = C.pointer(p)
            cmds[i].node_offset = off
            cmds[i].n_nodes = len(arr)
            cmds[i].opts = opts.to_abi()
            off += len(arr)
        nodes = np.ascontiguousarray(np.concatenate(arrays) if arrays else np.zeros(0, NODE_DTYPE))
        return nodes, cmds, keep

    def submit_new(self, fmt, w: int, h: int, fills: Sequence[Tuple[Pattern, object, FillOptions]],
                   init: Optional[np.ndarray] = None, out: Optional[np.ndarray] = None) -> int:
        """painter.fill for `fills` on a new w x h surface of `fmt` from the
        server's pool: initialised from `init` (z2d's byte layout) or cleared,
        and copied into `out` (a writable uint8 array of z2d's length) when
        the request completes."""
        f = abi.FORMAT_NAMES.index(fmt) if isinstance(fmt, str) else int(fmt)
        n = abi.surface_bytes(f, w, h)
        for a in (init, out):
            if a is not None and (a.dtype != np.uint8 or a.size < n or not a.flags["C_CONTIGUOUS"]):
                raise ValueError("init / out must be contiguous uint8 arrays of the surface's length")
        nodes, cmds, keep = self._pack(fills)
        t = C.c_uint64()
        check(self.lib.z2dgpu_server_submit_new(self.handle, f, w, h,
                                                None if init is None else init.ctypes.data_as(C.c_void_p),
                                                None if out is None else out.ctypes.data_as(C.c_void_p),
                                                nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(nodes), cmds,
                                                len(fills), C.byref(t)))
        if out is not None:
            self._outs[t.value] = out
        return t.value

    def submit(self, surface, fills: Sequence[Tuple[Pattern, object, FillOptions]]) -> int:
        keep: list = []
        arrays = []
        cmds = (abi.z2d_fill_cmd * max(1, len(fills)))()
        off = 0
        for i, (pat, nodes, opts) in enumerate(fills):
            arr = nodes if isinstance(nodes, np.ndarray) and nodes.dtype == NODE_DTYPE else None
            if arr is None:
                from .path import nodes_array
                arr = nodes_array(nodes)
            arrays.append(arr)
            p = pat.to_abi(keep)
            cmds[i].pattern = C.pointer(p)
            cmds[i].node_offset = off
            cmds[i].n_nodes = len(arr)
            cmds[i].opts = opts.to_abi()
            off += len(arr)
        nodes = np.ascontiguousarray(np.concatenate(arrays) if arrays else np.zeros(0, NODE_DTYPE))
        s = surface.to_abi()
        t = C.c_uint64()
        check(self.lib.z2dgpu_server_submit(self.handle, C.byref(s), nodes.ctypes.data_as(C.POINTER(abi.z2d_node)),
                                            len(nodes), cmds, len(fills), C.byref(t)))
        return t.value

    def submit_packed(self, surface_abi, nodes: np.ndarray, cmds: np.ndarray) -> int:
        """Raw entry: a z2d_surface, a NODE_DTYPE array and a z2d_fill_cmd
        array (z2d_gb300.batch.FILL_CMD_DTYPE) indexing it."""
        t = C.c_uint64()
        check(self.lib.z2dgpu_server_submit(self.handle, C.byref(surface_abi),
                                            nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(nodes),
                                            cmds.ctypes.data_as(C.POINTER(abi.z2d_fill_cmd)), len(cmds), C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> float:
        """Blocks until the request is drawn; returns its latency in µs
        (submit to completion).  Raises Z2DError (code ERR_TIMEOUT when
        timeout_ms ran out first)."""
        lat = C.c_double()
        rc = self.lib.z2dgpu_server_wait(self.handle, ticket, timeout_ms, C.byref(lat))
        if rc != abi.ERR_TIMEOUT:
            self._outs.pop(ticket, None)
        check(rc)
        return lat.value

    def info(self) -> dict:
        """All counters: batches, requests, deferred admissions, busy_ms,
        lanes, max_inflight (most batches drawn at once), pool_bytes,
        pool_peak_bytes."""
        st = abi.z2dgpu_server_stats_t()
        check(self.lib.z2dgpu_server_info(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def stats(self) -> Tuple[int, int, float]:
        b, r, ms = C.c_uint64(), C.c_uint64(), C.c_double()
        check(self.lib.z2dgpu_server_stats(self.handle, C.byref(b), C.byref(r), C.byref(ms)))
        return b.value, r.value, ms.value

    def close(self) -> None:
        if self.handle:
            self.lib.z2dgpu_server_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Server", "Z2DError"]
