"""ctypes binding and build recipe of the CPU oracle -- TEST INFRASTRUCTURE.

build_oracle() compiles z2d_oracle.cpp with g++ into oracle/_build/ (strict
IEEE flags: no FP contraction, no fast-math).  Oracle mirrors the product's
painter.fill / SurfaceCompositor.run entry points on host surfaces, using
the same C structs (include/z2dgpu.h).
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess
import threading

from z2d_gb300 import abi
from z2d_gb300.types import FillOptions, Operation, Pattern, nodes_to_abi

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "z2d_oracle.cpp"
SRC_STROKE = HERE / "z2d_stroke.cpp"
SRC_PATH = HERE / "z2d_path.cpp"
BUILD = HERE / "_build"
LIB = BUILD / "libz2doracle.so"
DEPS = [SRC, SRC_STROKE, SRC_PATH, HERE.parent / "include" / "z2dgpu.h", HERE.parent / "z2d_gb300" / "csrc" / "blue_noise_64x64.inc"]
CXXFLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]

_lock = threading.Lock()
_lib = None


def build_oracle(force: bool = False) -> pathlib.Path:
    """Compiles the oracle if it is missing or older than its sources."""
    BUILD.mkdir(exist_ok=True)
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in DEPS):
        return LIB
    tmp = BUILD / f"libz2doracle.{os.getpid()}.so"
    cmd = ["g++", *CXXFLAGS, "-o", str(tmp), str(SRC), str(SRC_STROKE), str(SRC_PATH)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def load_oracle():
    global _lib
    with _lock:
        if _lib is None:
            lib = C.CDLL(str(build_oracle()))
            lib.z2doracle_fill.argtypes = [C.POINTER(abi.z2d_surface), C.POINTER(abi.z2d_pattern),
                                           C.POINTER(abi.z2d_node), C.c_size_t, C.POINTER(abi.z2d_fill_opts)]
            lib.z2doracle_fill.restype = C.c_int
            lib.z2doracle_fill_contours.argtypes = [C.POINTER(abi.z2d_surface), C.POINTER(abi.z2d_pattern),
                                                    C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_size_t,
                                                    C.POINTER(abi.z2d_fill_opts)]
            lib.z2doracle_fill_contours.restype = C.c_int
            lib.z2doracle_hairline.argtypes = [C.POINTER(abi.z2d_surface), C.POINTER(abi.z2d_pattern),
                                               C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_size_t, C.c_int32,
                                               C.c_int32, C.c_int32]
            lib.z2doracle_hairline.restype = C.c_int
            lib.z2doracle_png_scanlines.argtypes = [C.POINTER(abi.z2d_surface), C.c_int32, C.c_void_p, C.c_size_t,
                                                    C.POINTER(C.c_size_t)]
            lib.z2doracle_png_scanlines.restype = C.c_int
            lib.z2doracle_composite.argtypes = [C.POINTER(abi.z2d_surface), C.c_int32, C.c_int32, C.c_int32,
                                                C.POINTER(abi.z2d_operation), C.c_int32]
            lib.z2doracle_composite.restype = C.c_int
            lib.z2doracle_run_pixel.argtypes = [C.c_int32, abi.z2d_pixel, abi.z2d_pixel, C.c_int32]
            lib.z2doracle_run_pixel.restype = abi.z2d_pixel
            lib.z2doracle_pixel_from_color.argtypes = [abi.z2d_color]
            lib.z2doracle_pixel_from_color.restype = abi.z2d_pixel
            lib.z2doracle_stroke_contours.argtypes = [C.POINTER(abi.z2d_node), C.c_size_t,
                                                      C.POINTER(abi.z2d_stroke_opts), C.c_int32,
                                                      C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_uint64),
                                                      C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_uint64),
                                                      C.POINTER(C.c_double)]
            lib.z2doracle_stroke_contours.restype = C.c_int
            lib.z2doracle_pow_f32.argtypes = [C.c_float, C.c_float]
            lib.z2doracle_pow_f32.restype = C.c_float
            lib.z2doracle_atan2.argtypes = [C.c_double, C.c_double]
            lib.z2doracle_atan2.restype = C.c_double
            lib.z2doracle_gradient_offset.argtypes = [C.POINTER(abi.z2d_gradient), C.c_int32, C.c_int32]
            lib.z2doracle_gradient_offset.restype = C.c_float
            lib.z2doracle_gradient_offsets.argtypes = [C.POINTER(abi.z2d_gradient), C.c_int32, C.c_int32, C.c_int32,
                                                       C.c_int32, C.c_void_p]
            lib.z2doracle_gradient_offsets.restype = None
            lib.z2doracle_build_paths.argtypes = [C.POINTER(abi.z2d_path_program), C.c_size_t,
                                                  C.POINTER(abi.z2d_path_cmd), C.c_size_t,
                                                  C.POINTER(abi.z2d_glyph_point), C.c_size_t, C.POINTER(C.c_uint16),
                                                  C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(C.c_uint64),
                                                  C.POINTER(C.c_int32)]
            lib.z2doracle_build_paths.restype = C.c_int
            lib.z2doracle_zig_trig.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_int)]
            lib.z2doracle_zig_trig.restype = C.c_double
            lib.z2doracle_gradient_pixel.argtypes = [C.POINTER(abi.z2d_gradient), C.c_int32, C.c_int32]
            lib.z2doracle_gradient_pixel.restype = abi.z2d_pixel
            lib.z2doracle_dither_pixel.argtypes = [C.POINTER(abi.z2d_pattern), C.c_int32, C.c_int32]
            lib.z2doracle_dither_pixel.restype = abi.z2d_pixel
            lib.z2doracle_plot.argtypes = [C.POINTER(abi.z2d_node), C.c_size_t, C.c_double, C.c_double,
                                           C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_double)]
            lib.z2doracle_plot.restype = C.c_int64
            lib.z2doracle_msaa_spans.argtypes = [C.c_uint32, C.POINTER(C.c_uint32), C.c_size_t,
                                                 C.POINTER(C.c_uint32), C.c_size_t]
            lib.z2doracle_msaa_spans.restype = C.c_uint32
            _lib = lib
    return _lib


def _host_abi(sfc) -> abi.z2d_surface:
    s = sfc.to_abi()
    if s.location != abi.MEM_HOST:
        raise ValueError("the oracle works on host surfaces only")
    return s


class Oracle:
    """painter.fill / SurfaceCompositor.run restated on the CPU."""

    def __init__(self):
        self.lib = load_oracle()

    def fill(self, surface, pattern: Pattern, nodes, opts: FillOptions = FillOptions()) -> int:
        keep: list = []
        s = _host_abi(surface)
        p = pattern.to_abi(keep)
        arr = nodes_to_abi(nodes)
        n = len(nodes)
        return self.lib.z2doracle_fill(C.byref(s), C.byref(p), arr, n, C.byref(opts.to_abi()))

    def fill_contours(self, surface, pattern: Pattern, contours, opts: FillOptions = FillOptions()) -> int:
        """The rasterisers on a polygon given as closed contours of
        already-scaled points (a list of (n, 2) arrays)."""
        import numpy as np
        keep: list = []
        s = _host_abi(surface)
        p = pattern.to_abi(keep)
        pts = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float64).reshape(-1, 2) for c in contours])
                                   if contours else np.zeros((1, 2)), dtype=np.float64)
        ends = np.cumsum([len(c) for c in contours]).astype(np.uint64) if contours else np.zeros(1, np.uint64)
        return self.lib.z2doracle_fill_contours(C.byref(s), C.byref(p), pts.ctypes.data_as(C.POINTER(C.c_double)),
                                                ends.ctypes.data_as(C.POINTER(C.c_uint64)), len(contours),
                                                C.byref(opts.to_abi()))

    def hairline(self, surface, pattern: Pattern, polylines, operator: str = "src_over", precision: str = "integer",
                 anti_aliasing: str = "default") -> int:
        """The hairline rasteriser on polylines (a list of (n, 2) arrays)."""
        import numpy as np
        keep: list = []
        s = _host_abi(surface)
        p = pattern.to_abi(keep)
        pts = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float64).reshape(-1, 2) for c in polylines])
                                   if polylines else np.zeros((1, 2)), dtype=np.float64)
        ends = np.cumsum([len(c) for c in polylines]).astype(np.uint64) if polylines else np.zeros(1, np.uint64)
        return self.lib.z2doracle_hairline(C.byref(s), C.byref(p), pts.ctypes.data_as(C.POINTER(C.c_double)),
                                           ends.ctypes.data_as(C.POINTER(C.c_uint64)), len(polylines),
                                           abi.OP[operator],
                                           {"integer": abi.PRECISION_INTEGER, "float": abi.PRECISION_FLOAT}[precision],
                                           {"none": abi.AA_NONE, "default": abi.AA_DEFAULT,
                                            "multisample_4x": abi.AA_MULTISAMPLE_4X,
                                            "supersample_4x": abi.AA_SUPERSAMPLE_4X}[anti_aliasing])

    def png_scanlines(self, surface, profile=None) -> bytes:
        """The PNG exporter's uncompressed image data for `surface`
        (profile None, "linear" or "srgb")."""
        import numpy as np
        s = _host_abi(surface)
        pr = {None: -1, "linear": 0, "srgb": 1}[profile]
        n = C.c_size_t()
        rc = self.lib.z2doracle_png_scanlines(C.byref(s), pr, None, 0, C.byref(n))
        if rc:
            raise RuntimeError(f"z2doracle_png_scanlines: {rc}")
        out = np.zeros(max(1, n.value), np.uint8)
        self.lib.z2doracle_png_scanlines(C.byref(s), pr, out.ctypes.data, n.value, C.byref(n))
        return out[:n.value].tobytes()

    def composite(self, dst, dst_x: int, dst_y: int, ops, precision: str = "integer") -> int:
        keep: list = []
        s = _host_abi(dst)
        arr = (abi.z2d_operation * max(1, len(ops)))()
        for i, o in enumerate(ops):
            arr[i] = o.to_abi(keep, _host_abi)
        prec = abi.PRECISION_FLOAT if precision == "float" else abi.PRECISION_INTEGER
        return self.lib.z2doracle_composite(C.byref(s), dst_x, dst_y, len(ops), arr, prec)

    def run_pixel(self, precision: str, dst, src, op: str):
        prec = abi.PRECISION_FLOAT if precision == "float" else abi.PRECISION_INTEGER
        return self.lib.z2doracle_run_pixel(prec, dst.to_abi(), src.to_abi(), abi.OP[op])

    def pixel_from_color(self, color):
        return self.lib.z2doracle_pixel_from_color(color.to_abi())

    def stroke_contours(self, nodes, opts, surface_format="rgba"):
        """The oracle's own stroke tessellation (z2d_stroke.cpp): the closed
        contours painter.stroke would rasterise on a surface of
        `surface_format` (hairlines: the open polylines), as a list of
        (n, 2) arrays of already-scaled points, and the rasteriser scale.
        Raises Z2DError with z2d's error on failure."""
        import numpy as np
        from z2d_gb300.native import Z2DError
        from z2d_gb300.types import _fmt
        keep: list = []
        arr = nodes_to_abi(nodes)
        o = opts.to_abi(keep)
        fmt = _fmt(surface_format)
        npts, nc, sc = C.c_uint64(), C.c_uint64(), C.c_double()
        rc = self.lib.z2doracle_stroke_contours(arr, len(nodes), C.byref(o), fmt, None, 0, C.byref(npts), None, 0,
                                                C.byref(nc), C.byref(sc))
        if rc:
            raise Z2DError(rc, "oracle stroke")
        pts = np.zeros(max(1, npts.value) * 2, np.float64)
        ends = np.zeros(max(1, nc.value), np.uint64)
        self.lib.z2doracle_stroke_contours(arr, len(nodes), C.byref(o), fmt, pts.ctypes.data_as(C.POINTER(C.c_double)),
                                           npts.value, C.byref(npts), ends.ctypes.data_as(C.POINTER(C.c_uint64)),
                                           nc.value, C.byref(nc), C.byref(sc))
        out, start = [], 0
        for e in ends[:nc.value]:
            out.append(pts[2 * start:2 * int(e)].reshape(-1, 2).copy())
            start = int(e)
        return out, sc.value

    def pow_f32(self, x: float, y: float) -> float:
        """std.math.pow(f32, x, y) as z2d computes it."""
        return self.lib.z2doracle_pow_f32(x, y)

    def atan2(self, y: float, x: float) -> float:
        """std.math.atan2(f64, y, x) as z2d computes it."""
        return self.lib.z2doracle_atan2(y, x)

    def gradient_offset(self, gradient, x: int, y: int) -> float:
        keep: list = []
        g = gradient.to_abi(keep)
        return self.lib.z2doracle_gradient_offset(C.byref(g), x, y)


    def zig_trig(self, which: str, x: float):
        """Zig's f64 sin / cos / tan as the oracle restates them (None beyond
        the medium argument range)."""
        ok = C.c_int()
        v = self.lib.z2doracle_zig_trig({"sin": 0, "cos": 1, "tan": 2}[which], x, C.byref(ok))
        return v if ok.value else None

    def build_paths(self, programs):
        """Path programs built by the oracle's Path restatement: (nodes per
        program as NODE_DTYPE arrays, status per program)."""
        from z2d_gb300.path_program import pack_programs, unpack_nodes
        packed = pack_programs(programs)
        return unpack_nodes(packed, lambda *a: self.lib.z2doracle_build_paths(*a))

    def gradient_offsets(self, gradient, x0: int, y0: int, w: int, h: int):
        """Gradient.getOffset for a w x h block of pixels (float32, row-major)."""
        import numpy as np
        keep = []
        g = gradient.to_abi(keep)
        out = np.empty((h, w), dtype=np.float32)
        self.lib.z2doracle_gradient_offsets(C.byref(g), x0, y0, w, h, out.ctypes.data)
        return out
    def gradient_pixel(self, gradient, x: int, y: int):
        keep: list = []
        g = gradient.to_abi(keep)
        return self.lib.z2doracle_gradient_pixel(C.byref(g), x, y)

    def dither_pixel(self, pattern: Pattern, x: int, y: int):
        keep: list = []
        p = pattern.to_abi(keep)
        return self.lib.z2doracle_dither_pixel(C.byref(p), x, y)

    def plot(self, nodes, scale: float, tolerance: float, cap: int = 1 << 16):
        arr = nodes_to_abi(nodes)
        out = (C.c_double * (4 * cap))()
        ext = (C.c_double * 4)()
        n = self.lib.z2doracle_plot(arr, len(nodes), scale, tolerance, out, cap, ext)
        if n < 0:
            return int(n), [], tuple(ext)
        edges = [tuple(out[4 * i: 4 * i + 4]) for i in range(min(n, cap))]
        return int(n), edges, tuple(ext)

    def msaa_spans(self, capacity: int, spans, cap: int = 4096):
        flat = (C.c_uint32 * max(1, 2 * len(spans)))(*[v for s in spans for v in s])
        out = (C.c_uint32 * (2 * cap))()
        n = self.lib.z2doracle_msaa_spans(capacity, flat, len(spans), out, cap)
        return int(n), [(out[2 * i], out[2 * i + 1]) for i in range(min(n, cap))]
