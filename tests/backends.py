"""Backends the scene restatements and parity tests drive: the GPU library
through its reference-shaped API, and the CPU oracle."""
from z2d_gb300 import abi
from z2d_gb300.native import Z2DError


class GpuBackend:
    """painter.fill / SurfaceCompositor.run through libz2dgpu.so."""

    def __init__(self, ctx=None):
        from z2d_gb300 import painter, compositor
        from z2d_gb300.native import default_context
        self.painter = painter
        self.compositor = compositor
        self.ctx = ctx or default_context()

    def fill(self, surface, pattern, nodes, opts):
        try:
            self.painter.fill(surface, pattern, nodes, opts, ctx=self.ctx)
        except Z2DError as e:
            return e.code
        return abi.OK

    def composite(self, dst, x, y, ops, precision="integer"):
        try:
            self.compositor.SurfaceCompositor.run(dst, x, y, ops, precision, ctx=self.ctx)
        except Z2DError as e:
            return e.code
        return abi.OK
