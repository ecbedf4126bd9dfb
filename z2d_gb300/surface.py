"""Surfaces: pixel buffers in z2d's in-memory layout, on the host or on the GPU.

Mirrors surface.Surface (src/surface.zig:74-351): eight pixel formats, 4 B/px
for ARGB/XRGB/RGB/RGBA, 1 B/px for alpha8 and LSB-first packed bits for
alpha4/2/1 with rows that are not byte aligned (flat index w*y+x).
"""
from __future__ import annotations

from typing import Optional, Union

import numpy as np

from . import abi
from .types import Pixel, _fmt


def _pixel_bytes(px: Pixel, fmt: int) -> np.ndarray:
    """T.fromPixel(px) (src/pixel.zig:399-433, 569-577) as the stored bytes
    of one pixel (ARGB/XRGB/RGB/RGBA/alpha8) or the raw packed value."""
    bits = abi.FORMAT_BITS
    colorful = (abi.FORMAT_ARGB, abi.FORMAT_XRGB, abi.FORMAT_RGB, abi.FORMAT_RGBA)
    has_alpha = (abi.FORMAT_ARGB, abi.FORMAT_RGBA, abi.FORMAT_ALPHA8, abi.FORMAT_ALPHA4,
                 abi.FORMAT_ALPHA2, abi.FORMAT_ALPHA1)

    def scale(v: int, frm: int, to: int) -> int:  # Alpha.scaleIntoIntAlpha, pixel.zig:582-626
        if frm == 1:
            return v * ((1 << to) - 1)
        if v == 0 or frm == to:
            return v
        if frm > to:
            return v >> (frm - to)
        d = to - frm
        if d in (2, 4):
            return (v << d) + v
        return (v << d) | (v << (to - 2 * frm)) | (v << (to - 3 * frm)) | v

    if fmt in colorful:
        if px.format in colorful:
            r, g, b = px.r, px.g, px.b
            a = px.a if px.format in has_alpha else 255
        else:
            r = g = b = 0
            a = scale(px.a, bits[px.format], 8)
        if fmt == abi.FORMAT_ARGB:
            return np.array([b, g, r, a], np.uint8)
        if fmt == abi.FORMAT_XRGB:
            return np.array([b, g, r, 0], np.uint8)
        if fmt == abi.FORMAT_RGB:
            return np.array([r, g, b, 0], np.uint8)
        return np.array([r, g, b, a], np.uint8)
    if px.format in (abi.FORMAT_XRGB, abi.FORMAT_RGB):
        v = (1 << bits[fmt]) - 1
    else:
        fb = 8 if px.format in colorful else bits[px.format]
        v = scale(px.a, fb, bits[fmt])
    return np.array([v], np.uint8)


class Surface:
    """A surface whose pixels live in host memory (numpy uint8 array) or in
    device memory (a torch uint8 CUDA tensor)."""

    def __init__(self, format: Union[int, str], width: int, height: int, data=None):
        self.format = _fmt(format)
        if width < 1:
            raise ValueError("InvalidWidth")
        if height < 1:
            raise ValueError("InvalidHeight")
        self.width = int(width)
        self.height = int(height)
        nbytes = abi.surface_bytes(self.format, self.width, self.height)
        if data is None:
            data = np.zeros(nbytes, np.uint8)
        if getattr(data, "numel", None) is not None:  # torch tensor
            # z2d's length, or (packed formats) padded to a 4-byte multiple
            padded = (nbytes + 3) // 4 * 4 if self.format >= abi.FORMAT_ALPHA4 else nbytes
            if data.numel() not in (nbytes, padded):
                raise ValueError(f"surface buffer has {data.numel()} bytes, need {nbytes}")
        elif data.size != nbytes:
            raise ValueError(f"surface buffer has {data.size} bytes, need {nbytes}")
        self.data = data

    # -- construction ------------------------------------------------------
    @staticmethod
    def init(format, width: int, height: int) -> "Surface":
        """Surface.init (src/surface.zig:97-123): zero-filled host surface."""
        return Surface(format, width, height)

    @staticmethod
    def init_pixel(px: Pixel, width: int, height: int, format=None) -> "Surface":
        """Surface.initPixel (src/surface.zig:128-152): surface of px's own
        format (or `format`) painted with px."""
        s = Surface(px.format if format is None else format, width, height)
        s.paint_pixel(px)
        return s

    def paint_pixel(self, px: Pixel) -> None:
        """paintPixel (src/surface.zig:525-527, 775-777, 890-915)."""
        v = _pixel_bytes(px, self.format)
        if self.format >= abi.FORMAT_ALPHA4:
            bits = abi.FORMAT_BITS[self.format]
            packed = 0
            for sh in range(0, 8 - bits + 1, bits):
                packed |= int(v[0]) << sh
            self._host()[:] = packed & 0xFF
        elif self.format == abi.FORMAT_ALPHA8:
            self._host()[:] = v[0]
        else:
            self._host().reshape(-1, 4)[:] = v

    def _host(self) -> np.ndarray:
        if not isinstance(self.data, np.ndarray):
            raise TypeError("operation needs a host surface")
        return self.data

    # -- location ----------------------------------------------------------
    @property
    def on_device(self) -> bool:
        return not isinstance(self.data, np.ndarray)

    def to_device(self, device: str = "cuda") -> "Surface":
        import torch
        h = np.ascontiguousarray(self.numpy())
        if self.format >= abi.FORMAT_ALPHA4:  # pad to a 4-byte multiple (word atomics)
            h = np.concatenate([h, np.zeros((-h.size) % 4, np.uint8)])
        t = torch.from_numpy(h).to(device)
        return Surface(self.format, self.width, self.height, t)

    def to_host(self) -> "Surface":
        return Surface(self.format, self.width, self.height, self.numpy().copy())

    def numpy(self) -> np.ndarray:
        if isinstance(self.data, np.ndarray):
            return self.data
        nbytes = abi.surface_bytes(self.format, self.width, self.height)
        return self.data.detach().cpu().numpy()[:nbytes]

    def copy(self) -> "Surface":
        if isinstance(self.data, np.ndarray):
            return Surface(self.format, self.width, self.height, self.data.copy())
        return Surface(self.format, self.width, self.height, self.data.clone())

    def to_abi(self) -> abi.z2d_surface:
        s = abi.z2d_surface()
        s.format, s.width, s.height = self.format, self.width, self.height
        if isinstance(self.data, np.ndarray):
            if not self.data.flags["C_CONTIGUOUS"]:
                raise ValueError("surface data must be contiguous")
            s.location = abi.MEM_HOST
            s.data = self.data.ctypes.data
        else:
            if not self.data.is_contiguous():
                raise ValueError("surface data must be contiguous")
            s.location = abi.MEM_DEVICE
            s.data = self.data.data_ptr()
        return s

    # -- pixel access (tests, export) ---------------------------------------
    def pixels(self) -> np.ndarray:
        """Per-pixel view: (h, w, 4) uint8 for 32-bit formats (stored byte
        order), (h, w) raw values for alpha formats."""
        d = self.numpy()
        if self.format <= abi.FORMAT_RGBA:
            return d.reshape(self.height, self.width, 4)
        if self.format == abi.FORMAT_ALPHA8:
            return d.reshape(self.height, self.width)
        bits = abi.FORMAT_BITS[self.format]
        per = 8 // bits
        idx = np.arange(self.width * self.height)
        vals = (d[idx // per] >> ((idx % per) * bits).astype(np.uint8)) & ((1 << bits) - 1)
        return vals.reshape(self.height, self.width).astype(np.uint8)

    def get_pixel(self, x: int, y: int) -> Optional[Pixel]:
        if x < 0 or y < 0 or x >= self.width or y >= self.height:
            return None
        p = self.pixels()
        f = self.format
        if f == abi.FORMAT_ARGB:
            b, g, r, a = p[y, x]
            return Pixel.argb(int(r), int(g), int(b), int(a))
        if f == abi.FORMAT_XRGB:
            b, g, r, _ = p[y, x]
            return Pixel.xrgb(int(r), int(g), int(b))
        if f == abi.FORMAT_RGB:
            r, g, b, _ = p[y, x]
            return Pixel.rgb(int(r), int(g), int(b))
        if f == abi.FORMAT_RGBA:
            r, g, b, a = p[y, x]
            return Pixel.rgba(int(r), int(g), int(b), int(a))
        return Pixel(f, 0, 0, 0, int(p[y, x]))
