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

    def stroke(self, surface, pattern, nodes, opts):
        try:
            self.painter.stroke(surface, pattern, nodes, opts, ctx=self.ctx)
        except Z2DError as e:
            return e.code
        return abi.OK


class StrokeOracle:
    """The oracle with painter.stroke: the stroke polygon (or hairline
    polylines) comes from the oracle's own restatement of z2d's stroke
    tessellation (oracle/z2d_stroke.cpp, pinned to z2d by the stroke scenes'
    golden PNGs) and is rasterised by the oracle; nothing of the library
    takes part."""

    def __init__(self, oracle):
        self.oracle = oracle

    def fill(self, surface, pattern, nodes, opts):
        return self.oracle.fill(surface, pattern, nodes, opts)

    def composite(self, dst, x, y, ops, precision="integer"):
        return self.oracle.composite(dst, x, y, ops, precision)

    def stroke(self, surface, pattern, nodes, opts):
        from z2d_gb300.types import FillOptions
        try:
            contours, _ = self.oracle.stroke_contours(nodes, opts, surface.format)
        except Z2DError as e:
            return e.code
        if opts.hairline:  # polylines of polyline_plotter, drawn by the hairline rasteriser
            return self.oracle.hairline(surface, pattern, contours, opts.operator, opts.precision, opts.anti_aliasing)
        aa = "none" if surface.format == abi.FORMAT_ALPHA1 else opts.anti_aliasing
        fo = FillOptions(anti_aliasing=aa, fill_rule="non_zero", operator=opts.operator, precision=opts.precision)
        return self.oracle.fill_contours(surface, pattern, contours, fo)
