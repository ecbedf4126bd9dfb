"""Request queue in front of the multi-surface fill pass (z2dgpu_server_*).

    srv = Server(max_batch_jobs=256, max_wait_us=200)
    t = srv.submit(surface, [(pattern, nodes, opts), ...])   # any thread
    latency_us = srv.wait(t)                                 # raises Z2DError on failure
    srv.close()

Surfaces must be device-resident (Surface.to_device) and stay alive until
their requests complete.  Requests on one surface are drawn in submission
order.  There is no counterpart in z2d: it is the serving loop around
painter.fill.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from . import abi
from .native import Z2DError, check, load
from .types import NODE_DTYPE, FillOptions, Pattern


class Server:
    def __init__(self, device: int = 0, max_batch_jobs: int = 256, max_wait_us: int = 200):
        self.lib = load()
        self.handle = C.c_void_p()
        check(self.lib.z2dgpu_server_create(C.byref(self.handle), device, max_batch_jobs, max_wait_us))

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
        check(self.lib.z2dgpu_server_wait(self.handle, ticket, timeout_ms, C.byref(lat)))
        return lat.value

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
