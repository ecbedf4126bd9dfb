"""ctypes mirror of include/z2dgpu.h (the C ABI of the fill/composite path).

The struct layouts and enum values here must match the header exactly; the
header cites the z2d interfaces each one replaces.
"""
from __future__ import annotations

import ctypes as C

# status codes (src/painter.zig:54-63, src/surface.zig:85-91)
OK = 0
ERR_PATH_NOT_CLOSED = 1
ERR_PIXEL_NOT_PREMULTIPLIED = 2
ERR_INVALID_DIMENSIONS = 3
ERR_INVALID_STATE = 4
ERR_OUT_OF_MEMORY = 5
ERR_CUDA = 6
ERR_TIMEOUT = 7
ERR_INVALID_ARGUMENT = 8

# pixel formats (src/pixel.zig:47-56)
FORMAT_ARGB, FORMAT_XRGB, FORMAT_RGB, FORMAT_RGBA = 0, 1, 2, 3
FORMAT_ALPHA8, FORMAT_ALPHA4, FORMAT_ALPHA2, FORMAT_ALPHA1 = 4, 5, 6, 7
FORMAT_NAMES = ["argb", "xrgb", "rgb", "rgba", "alpha8", "alpha4", "alpha2", "alpha1"]
FORMAT_BITS = [32, 32, 32, 32, 8, 4, 2, 1]

MEM_HOST, MEM_DEVICE = 0, 1

# operators (src/compositor.zig:46-158), same order
OPERATORS = [
    "clear", "src", "dst", "src_over", "dst_over", "src_in", "dst_in", "src_out",
    "dst_out", "src_atop", "dst_atop", "xor", "plus", "multiply", "screen",
    "overlay", "darken", "lighten", "color_dodge", "color_burn", "hard_light",
    "soft_light", "difference", "exclusion", "hue", "saturation", "color",
    "luminosity",
]
OP = {name: i for i, name in enumerate(OPERATORS)}
FLOAT_ONLY_OPS = {"color_dodge", "color_burn", "soft_light", "hue", "saturation", "color", "luminosity"}
UNBOUNDED_OPS = {"src_in", "dst_in", "src_out", "dst_atop"}

PRECISION_INTEGER, PRECISION_FLOAT = 0, 1
FILL_NON_ZERO, FILL_EVEN_ODD = 0, 1
AA_NONE, AA_DEFAULT, AA_MULTISAMPLE_4X, AA_SUPERSAMPLE_4X = 0, 1, 2, 3

MOVE_TO, LINE_TO, CURVE_TO, CLOSE_PATH = 0, 1, 2, 3

COLOR_LINEAR_RGB, COLOR_SRGB, COLOR_HSL = 0, 1, 2
GRADIENT_LINEAR, GRADIENT_RADIAL, GRADIENT_CONIC = 0, 1, 2
INTERP_LINEAR_RGB, INTERP_SRGB = 0, 1
INTERP_HSL = {"shorter": 2, "longer": 3, "increasing": 4, "decreasing": 5}

PATTERN_PIXEL, PATTERN_GRADIENT, PATTERN_DITHER = 0, 1, 2
DITHER_NONE, DITHER_BAYER, DITHER_BLUE_NOISE = 0, 1, 2
DITHER_SRC_PIXEL, DITHER_SRC_COLOR, DITHER_SRC_GRADIENT = 0, 1, 2

PARAM_NONE, PARAM_PIXEL, PARAM_GRADIENT, PARAM_DITHER, PARAM_SURFACE = 0, 1, 2, 3, 4


class z2d_pixel(C.Structure):
    _fields_ = [("format", C.c_int32), ("r", C.c_uint8), ("g", C.c_uint8),
                ("b", C.c_uint8), ("a", C.c_uint8)]


class z2dgpu_server_opts(C.Structure):
    _fields_ = [("max_batch_jobs", C.c_int32), ("max_wait_us", C.c_int32), ("lanes", C.c_int32),
                ("pool_bytes", C.c_int64)]


class z2dgpu_server_stats_t(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("requests", C.c_uint64), ("deferred", C.c_uint64), ("busy_ms", C.c_double),
                ("lanes", C.c_int32), ("max_inflight", C.c_int32), ("pool_bytes", C.c_int64),
                ("pool_peak_bytes", C.c_int64)]


class z2d_surface(C.Structure):
    _fields_ = [("format", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("location", C.c_int32), ("data", C.c_void_p)]


class z2d_node(C.Structure):
    _fields_ = [("tag", C.c_int32), ("_pad", C.c_int32), ("p", C.c_double * 6)]


# path programs (include/z2dgpu.h: z2dgpu_build_paths)
(PATH_MOVE_TO, PATH_LINE_TO, PATH_CURVE_TO, PATH_REL_MOVE_TO, PATH_REL_LINE_TO, PATH_REL_CURVE_TO, PATH_ARC,
 PATH_ARC_NEGATIVE, PATH_CLOSE, PATH_SET_TRANSFORMATION, PATH_SET_TOLERANCE, PATH_RESET, PATH_GLYPH) = range(13)


class z2d_path_cmd(C.Structure):
    _fields_ = [("op", C.c_int32), ("_pad", C.c_int32), ("v", C.c_double * 6)]


class z2d_path_program(C.Structure):
    _fields_ = [("cmd_offset", C.c_uint64), ("n_cmds", C.c_uint64), ("transformation", C.c_double * 6),
                ("tolerance", C.c_double)]


class z2d_glyph_point(C.Structure):
    _fields_ = [("x", C.c_int16), ("y", C.c_int16), ("flags", C.c_uint16), ("_pad", C.c_uint16)]


class z2d_color(C.Structure):
    _fields_ = [("space", C.c_int32), ("c", C.c_float * 4)]


class z2d_stop(C.Structure):
    _fields_ = [("offset", C.c_float), ("color", z2d_color)]


class z2d_gradient(C.Structure):
    _fields_ = [("type", C.c_int32), ("method", C.c_int32), ("n_stops", C.c_int32),
                ("_pad", C.c_int32), ("geom", C.c_double * 6),
                ("transform", C.c_double * 6), ("stops", C.POINTER(z2d_stop))]


class z2d_pattern(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pixel", z2d_pixel),
                ("gradient", C.POINTER(z2d_gradient)), ("dither_type", C.c_int32),
                ("dither_source", C.c_int32), ("dither_scale", C.c_int32),
                ("_pad", C.c_int32), ("dither_color", z2d_color)]


class z2d_fill_opts(C.Structure):
    _fields_ = [("anti_aliasing", C.c_int32), ("fill_rule", C.c_int32), ("op", C.c_int32),
                ("precision", C.c_int32), ("tolerance", C.c_double)]


class z2d_param(C.Structure):
    _fields_ = [("kind", C.c_int32), ("_pad", C.c_int32), ("pattern", z2d_pattern),
                ("surface", C.POINTER(z2d_surface))]


class z2d_operation(C.Structure):
    _fields_ = [("op", C.c_int32), ("_pad", C.c_int32), ("dst", z2d_param), ("src", z2d_param)]


class z2d_fill_cmd(C.Structure):
    _fields_ = [("pattern", C.POINTER(z2d_pattern)), ("node_offset", C.c_uint64),
                ("n_nodes", C.c_uint64), ("opts", z2d_fill_opts)]


JOIN_MITER, JOIN_ROUND, JOIN_BEVEL = 0, 1, 2
CAP_BUTT, CAP_ROUND, CAP_SQUARE = 0, 1, 2


class z2d_stroke_opts(C.Structure):
    _fields_ = [("anti_aliasing", C.c_int32), ("line_join", C.c_int32), ("line_cap", C.c_int32), ("op", C.c_int32),
                ("precision", C.c_int32), ("hairline", C.c_int32), ("line_width", C.c_double),
                ("miter_limit", C.c_double), ("tolerance", C.c_double), ("dash_offset", C.c_double),
                ("transformation", C.c_double * 6), ("dashes", C.POINTER(C.c_double)), ("n_dashes", C.c_uint64)]


DRAW_FILL, DRAW_STROKE = 0, 1


class z2d_draw_cmd(C.Structure):
    _fields_ = [("kind", C.c_int32), ("_pad", C.c_int32), ("pattern", C.POINTER(z2d_pattern)),
                ("node_offset", C.c_uint64), ("n_nodes", C.c_uint64), ("fill", z2d_fill_opts),
                ("stroke", z2d_stroke_opts)]


class z2d_job(C.Structure):
    _fields_ = [("surface", z2d_surface), ("cmd_offset", C.c_uint64), ("n_cmds", C.c_uint64)]


def surface_bytes(fmt: int, width: int, height: int) -> int:
    """Storage size of a surface (src/surface.zig:382-395, 621-635)."""
    return (width * height * FORMAT_BITS[fmt] + 7) // 8


# Every symbol include/z2dgpu.h declares (checked by the ABI tests).
EXPORTED_SYMBOLS = [
    "z2dgpu_version", "z2dgpu_last_error", "z2dgpu_ctx_create", "z2dgpu_ctx_destroy",
    "z2dgpu_ctx_synchronize", "z2dgpu_ctx_launch_count", "z2dgpu_ctx_set_timing",
    "z2dgpu_ctx_kernel_ms", "z2dgpu_ctx_set_raster", "z2dgpu_ctx_raster_tuning", "z2dgpu_surface_bytes",
    "z2dgpu_fill", "z2dgpu_fill_batch", "z2dgpu_fill_jobs", "z2dgpu_draw_jobs", "z2dgpu_stroke",
    "z2dgpu_stroke_contours",
    "z2dgpu_composite",
    "z2dgpu_composite_noalloc", "z2dgpu_server_create", "z2dgpu_server_submit", "z2dgpu_server_wait",
    "z2dgpu_server_stats", "z2dgpu_server_destroy", "z2dgpu_server_create2", "z2dgpu_server_submit_new",
    "z2dgpu_server_info", "z2dgpu_png_encode", "z2dgpu_png_scanlines", "z2dgpu_free", "z2dgpu_gradient_offsets", "z2dgpu_build_paths",
]

PROFILE = {None: -1, "linear": 0, "srgb": 1}  # color.RGBProfile of the PNG exporter
