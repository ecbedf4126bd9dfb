"""Loads libz2dgpu.so (building it in-tree when missing) and declares the C
ABI of include/z2dgpu.h.  There is no fallback: if the library cannot be
built or loaded, every entry point raises."""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import abi

_lock = threading.Lock()
_lib = None


class Z2DError(RuntimeError):
    """A non-zero status from the C ABI (codes mirror z2d's error sets)."""

    NAMES = {
        abi.ERR_PATH_NOT_CLOSED: "PathNotClosed",
        abi.ERR_PIXEL_NOT_PREMULTIPLIED: "PixelSourceNotPreMultiplied",
        abi.ERR_INVALID_DIMENSIONS: "InvalidDimensions",
        abi.ERR_INVALID_STATE: "InvalidState",
        abi.ERR_OUT_OF_MEMORY: "OutOfMemory",
        abi.ERR_CUDA: "CudaError",
        abi.ERR_TIMEOUT: "Timeout",
        abi.ERR_INVALID_ARGUMENT: "InvalidArgument",
    }

    def __init__(self, code: int, message: str = ""):
        self.code = code
        super().__init__(f"{self.NAMES.get(code, code)}: {message}")


def library_path() -> str:
    from .build import LIB
    return str(LIB)


def load(build_if_missing: bool = True):
    """Returns the loaded library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if build_if_missing and not os.environ.get("Z2D_NO_BUILD"):
            from .build import build
            build()
        if not os.path.exists(path):
            raise RuntimeError(f"libz2dgpu.so is missing ({path}); run z2d_gb300.build")
        lib = C.CDLL(path)
        P = C.POINTER
        lib.z2dgpu_version.restype = C.c_char_p
        lib.z2dgpu_last_error.restype = C.c_char_p
        lib.z2dgpu_ctx_create.argtypes = [P(C.c_void_p), C.c_int, C.c_void_p]
        lib.z2dgpu_ctx_destroy.argtypes = [C.c_void_p]
        lib.z2dgpu_ctx_synchronize.argtypes = [C.c_void_p]
        lib.z2dgpu_ctx_launch_count.argtypes = [C.c_void_p]
        lib.z2dgpu_ctx_launch_count.restype = C.c_uint64
        lib.z2dgpu_ctx_set_timing.argtypes = [C.c_void_p, C.c_int]
        lib.z2dgpu_ctx_set_timing.restype = C.c_int
        lib.z2dgpu_ctx_set_raster.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
        lib.z2dgpu_ctx_set_raster.restype = C.c_int
        lib.z2dgpu_ctx_raster_tuning.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32), P(C.c_int32), P(C.c_int32)]
        lib.z2dgpu_ctx_raster_tuning.restype = C.c_int
        lib.z2dgpu_ctx_kernel_ms.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_uint64)]
        lib.z2dgpu_ctx_kernel_ms.restype = C.c_double
        lib.z2dgpu_surface_bytes.argtypes = [C.c_int32, C.c_int32, C.c_int32]
        lib.z2dgpu_surface_bytes.restype = C.c_size_t
        lib.z2dgpu_fill.argtypes = [C.c_void_p, P(abi.z2d_surface), P(abi.z2d_pattern), P(abi.z2d_node), C.c_size_t,
                                    P(abi.z2d_fill_opts)]
        lib.z2dgpu_fill_batch.argtypes = [C.c_void_p, P(abi.z2d_surface), P(abi.z2d_node), C.c_size_t,
                                          P(abi.z2d_fill_cmd), C.c_size_t]
        lib.z2dgpu_stroke.argtypes = [C.c_void_p, P(abi.z2d_surface), P(abi.z2d_pattern), P(abi.z2d_node), C.c_size_t,
                                      P(abi.z2d_stroke_opts)]
        lib.z2dgpu_stroke_contours.argtypes = [P(abi.z2d_node), C.c_size_t, P(abi.z2d_stroke_opts), C.c_int32,
                                               P(C.c_double), C.c_size_t, P(C.c_uint64), P(C.c_uint64), C.c_size_t,
                                               P(C.c_uint64), P(C.c_double)]
        lib.z2dgpu_stroke.restype = C.c_int
        lib.z2dgpu_draw_jobs.argtypes = [C.c_void_p, P(abi.z2d_job), C.c_size_t, P(abi.z2d_node), C.c_size_t,
                                         P(abi.z2d_draw_cmd), C.c_size_t]
        lib.z2dgpu_draw_jobs.restype = C.c_int
        lib.z2dgpu_stroke_contours.restype = C.c_int
        lib.z2dgpu_fill_jobs.argtypes = [C.c_void_p, P(abi.z2d_job), C.c_size_t, P(abi.z2d_node), C.c_size_t,
                                         P(abi.z2d_fill_cmd), C.c_size_t]
        lib.z2dgpu_composite.argtypes = [C.c_void_p, P(abi.z2d_surface), C.c_int32, C.c_int32, C.c_int32,
                                         P(abi.z2d_operation), C.c_int32]
        lib.z2dgpu_composite_noalloc.argtypes = [C.c_int, C.c_void_p, P(abi.z2d_surface), C.c_int32, C.c_int32,
                                                 C.c_int32, P(abi.z2d_operation), C.c_int32]
        lib.z2dgpu_server_create.argtypes = [P(C.c_void_p), C.c_int, C.c_int32, C.c_int32]
        lib.z2dgpu_server_create2.argtypes = [P(C.c_void_p), C.c_int, P(abi.z2dgpu_server_opts)]
        lib.z2dgpu_server_submit_new.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                                 P(abi.z2d_node), C.c_size_t, P(abi.z2d_fill_cmd), C.c_size_t,
                                                 P(C.c_uint64)]
        lib.z2dgpu_server_info.argtypes = [C.c_void_p, P(abi.z2dgpu_server_stats_t)]
        lib.z2dgpu_server_submit.argtypes = [C.c_void_p, P(abi.z2d_surface), P(abi.z2d_node), C.c_size_t,
                                             P(abi.z2d_fill_cmd), C.c_size_t, P(C.c_uint64)]
        lib.z2dgpu_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_int32, P(C.c_double)]
        lib.z2dgpu_server_stats.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_uint64), P(C.c_double)]
        lib.z2dgpu_server_destroy.argtypes = [C.c_void_p]
        for name in ("z2dgpu_png_encode", "z2dgpu_png_scanlines"):
            getattr(lib, name).argtypes = [C.c_void_p, P(abi.z2d_surface), C.c_int32, P(P(C.c_uint8)),
                                           P(C.c_size_t)]
            getattr(lib, name).restype = C.c_int
        lib.z2dgpu_free.argtypes = [C.c_void_p]
        lib.z2dgpu_free.restype = None
        lib.z2dgpu_gradient_offsets.argtypes = [C.c_void_p, P(abi.z2d_gradient), C.c_int32, C.c_int32, C.c_int32,
                                                C.c_int32, C.c_void_p, P(C.c_int64)]
        lib.z2dgpu_gradient_offsets.restype = C.c_int
        lib.z2dgpu_build_paths.argtypes = [C.c_void_p, P(abi.z2d_path_program), C.c_size_t, P(abi.z2d_path_cmd),
                                           C.c_size_t, P(abi.z2d_glyph_point), C.c_size_t, P(C.c_uint16),
                                           C.c_size_t, C.c_void_p, C.c_size_t, P(C.c_uint64), P(C.c_int32)]
        lib.z2dgpu_build_paths.restype = C.c_int
        for name in ("z2dgpu_server_create", "z2dgpu_server_create2", "z2dgpu_server_submit",
                     "z2dgpu_server_submit_new", "z2dgpu_server_wait", "z2dgpu_server_stats", "z2dgpu_server_info",
                     "z2dgpu_server_destroy"):
            getattr(lib, name).restype = C.c_int
        for name in ("z2dgpu_ctx_create", "z2dgpu_ctx_destroy", "z2dgpu_ctx_synchronize", "z2dgpu_fill",
                     "z2dgpu_fill_batch", "z2dgpu_fill_jobs", "z2dgpu_composite", "z2dgpu_composite_noalloc"):
            getattr(lib, name).restype = C.c_int
        _lib = lib
        return lib


def check(rc: int) -> int:
    if rc != abi.OK:
        msg = load().z2dgpu_last_error().decode(errors="replace")
        raise Z2DError(rc, msg)
    return rc


class Context:
    """A z2dgpu_ctx: one CUDA stream plus reusable device scratch."""

    def __init__(self, device: int = 0, stream=None):
        self.lib = load()
        h = C.c_void_p()
        s = None
        if stream is not None:
            s = C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))
        check(self.lib.z2dgpu_ctx_create(C.byref(h), device, s))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.z2dgpu_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        check(self.lib.z2dgpu_ctx_synchronize(self.handle))

    def set_timing(self, enable: bool) -> None:
        check(self.lib.z2dgpu_ctx_set_timing(self.handle, 1 if enable else 0))

    def set_raster(self, ctas_per_sm: int = -2, order: int = 0, tile_items: int = 1) -> None:
        """Forces the rasteriser's schedule (grid: -1 = one CTA per tile, 0 =
        persistent with as many resident CTAs as fit, n = n per SM; queue
        order 0 = tiles in order, 1 = bands with the most fills first; queue
        item 1 = a tile per CTA, 0 = a tile row per warp); ctas_per_sm = -2
        returns to the autotuner."""
        check(self.lib.z2dgpu_ctx_set_raster(self.handle, ctas_per_sm, order, tile_items))

    def raster_tuning(self) -> dict:
        """The autotuner's state for the last pass drawn on this context."""
        d, ct, od, it = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        check(self.lib.z2dgpu_ctx_raster_tuning(self.handle, C.byref(d), C.byref(ct), C.byref(od), C.byref(it)))
        return {"decided": d.value, "ctas_per_sm": ct.value, "order": od.value, "tile_items": it.value}

    def gradient_offsets(self, gradient, x0: int, y0: int, w: int, h: int):
        """The offsets the kernels evaluate for a w x h block of pixels
        (float32, row-major) and how many took the f64 code."""
        import numpy as np
        keep: list = []
        g = gradient.to_abi(keep)
        out = np.empty((h, w), dtype=np.float32)
        n = C.c_int64()
        check(self.lib.z2dgpu_gradient_offsets(self.handle, C.byref(g), x0, y0, w, h, out.ctypes.data, C.byref(n)))
        return out, int(n.value)

    def kernel_ms(self, kernel: str):
        n = C.c_uint64()
        ms = self.lib.z2dgpu_ctx_kernel_ms(self.handle, kernel.encode(), C.byref(n))
        return float(ms), int(n.value)

    @property
    def launch_count(self) -> int:
        return int(self.lib.z2dgpu_ctx_launch_count(self.handle))


_default_ctx = {}


def default_context(device: int = 0) -> Context:
    ctx = _default_ctx.get(device)
    if ctx is None:
        ctx = Context(device)
        _default_ctx[device] = ctx
    return ctx
