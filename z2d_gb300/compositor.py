"""compositor.SurfaceCompositor with z2d's interface, running on the GPU.

SurfaceCompositor.run (src/compositor.zig:302-440) and Surface.composite
(src/surface.zig:225-241).  Batches of 1 or 2 operations.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

from . import abi
from .native import Context, check, default_context
from .types import Operation


class SurfaceCompositor:
    @staticmethod
    def run(dst, dst_x: int, dst_y: int, operations: Sequence[Operation], precision: str = "integer",
            ctx: Optional[Context] = None) -> None:
        ctx = ctx or default_context()
        keep: list = []
        arr = (abi.z2d_operation * max(1, len(operations)))()
        for i, o in enumerate(operations):
            arr[i] = o.to_abi(keep, lambda s: s.to_abi())
        d = dst.to_abi()
        prec = abi.PRECISION_FLOAT if precision == "float" else abi.PRECISION_INTEGER
        check(ctx.lib.z2dgpu_composite(ctx.handle, C.byref(d), dst_x, dst_y, len(operations), arr, prec))


def composite(dst, src, operator: str, dst_x: int, dst_y: int, precision: str = "integer",
              ctx: Optional[Context] = None) -> None:
    """Surface.composite: one operation with a surface source."""
    SurfaceCompositor.run(dst, dst_x, dst_y, [Operation(operator, src=src)], precision, ctx)


def run_noalloc(dst, dst_x: int, dst_y: int, operations: Sequence[Operation], precision: str = "integer",
                device: int = 0, stream: int = 0) -> None:
    """SurfaceCompositor.run through z2dgpu_composite_noalloc, for callers
    that may not allocate device memory while compositing (the library
    never allocates in this call).  `dst` and every surface param must be
    on `device`; the work is queued on the raw CUDA stream handle `stream`
    (0 = the default stream).  At most 4 gradient params per call; calls
    whose GPU work overlaps race on the library's shared gradient array."""
    from .native import load
    lib = load()
    keep: list = []
    arr = (abi.z2d_operation * max(1, len(operations)))()
    for i, o in enumerate(operations):
        arr[i] = o.to_abi(keep, lambda s: s.to_abi())
    d = dst.to_abi()
    prec = abi.PRECISION_FLOAT if precision == "float" else abi.PRECISION_INTEGER
    check(lib.z2dgpu_composite_noalloc(device, C.c_void_p(stream), C.byref(d), dst_x, dst_y, len(operations), arr,
                                       prec))
