"""PNG export (z2d's png_exporter, src/export_png.zig) through the GPU
encoder: z2dgpu_png_encode / z2dgpu_png_scanlines."""
from __future__ import annotations

import ctypes as C
from typing import Optional

from . import abi
from .native import check, default_context, Context


def _call(fn_name: str, surface, color_profile: Optional[str], ctx: Optional[Context]) -> bytes:
    ctx = ctx or default_context()
    out = C.POINTER(C.c_uint8)()
    n = C.c_size_t()
    keep: list = []
    s = surface.to_abi() if hasattr(surface, "to_abi") else surface
    keep.append(s)
    check(getattr(ctx.lib, fn_name)(ctx.handle, C.byref(s), abi.PROFILE[color_profile], C.byref(out), C.byref(n)))
    try:
        return C.string_at(out, n.value)
    finally:
        ctx.lib.z2dgpu_free(out)


def encode(surface, color_profile: Optional[str] = None, ctx: Optional[Context] = None) -> bytes:
    """The PNG file writeToPNGFile would write for `surface` (host or
    device memory); color_profile None, "linear" or "srgb"."""
    return _call("z2dgpu_png_encode", surface, color_profile, ctx)


def scanlines(surface, color_profile: Optional[str] = None, ctx: Optional[Context] = None) -> bytes:
    """The PNG's uncompressed image data: per row a 0 filter byte and the
    encoded pixels."""
    return _call("z2dgpu_png_scanlines", surface, color_profile, ctx)


def write_to_png_file(surface, filename: str, color_profile: Optional[str] = None,
                      ctx: Optional[Context] = None) -> None:
    """png_exporter.writeToPNGFile (src/export_png.zig:56-87)."""
    with open(filename, "wb") as f:
        f.write(encode(surface, color_profile, ctx))
