"""Minimal PNG reader and z2d export transform for golden comparisons.

z2d's exporter (src/export_png.zig:97-371) writes RGB/RGBA at 8 bits with
RGBA demultiplied, alpha surfaces as grey at 8/4/2/1 bits packed MSB-first
per row, and optionally applies sRGB gamma.  Goldens are compared by decoded
pixels after applying the same transform to our surface, not by file bytes
(the zlib stream differs).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

from z2d_gb300 import abi


def read_png(path: str):
    """Returns (width, height, bit_depth, color_type, rows) where rows is a
    list of unfiltered scanline byte strings."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos = 8
    idat = b""
    ihdr = None
    while pos < len(data):
        (ln,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
    w, h, depth, ctype, _, _, interlace = ihdr
    assert interlace == 0
    raw = zlib.decompress(idat)
    chans = {0: 1, 2: 3, 6: 4}[ctype]
    bpp = max(1, chans * depth // 8)
    stride = (w * chans * depth + 7) // 8
    rows = []
    prev = bytearray(stride)
    p = 0
    for _ in range(h):
        ft = raw[p]
        line = bytearray(raw[p + 1:p + 1 + stride])
        p += 1 + stride
        for i in range(stride):
            a = line[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ft == 1:
                line[i] = (line[i] + a) & 0xFF
            elif ft == 2:
                line[i] = (line[i] + b) & 0xFF
            elif ft == 3:
                line[i] = (line[i] + ((a + b) >> 1)) & 0xFF
            elif ft == 4:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                line[i] = (line[i] + pr) & 0xFF
        rows.append(bytes(line))
        prev = line
    return w, h, depth, ctype, rows


def png_chunks(data: bytes):
    """(type, body) of every chunk, checking each CRC."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, out = 8, []
    while pos < len(data):
        (ln,) = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + ln]
        (crc,) = struct.unpack(">I", data[pos + 8 + ln:pos + 12 + ln])
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == crc, f"bad CRC in {typ}"
        out.append((typ, body))
        pos += 12 + ln
    return out


def golden_scanlines(path: str) -> bytes:
    """The PNG's decompressed image data (filter bytes included)."""
    chunks = png_chunks(open(path, "rb").read())
    return zlib.decompress(b"".join(body for typ, body in chunks if typ == b"IDAT"))


def golden_pixels(path: str) -> np.ndarray:
    """Decoded golden as (h, w, c) uint8 values (c = 1 for grey)."""
    w, h, depth, ctype, rows = read_png(path)
    if depth == 8:
        chans = {0: 1, 2: 3, 6: 4}[ctype]
        arr = np.frombuffer(b"".join(rows), np.uint8).reshape(h, w, chans)
        return arr
    per = 8 // depth
    out = np.zeros((h, w, 1), np.uint8)
    for y, row in enumerate(rows):
        for x in range(w):
            byte = row[x // per]
            sh = 8 - depth - (x % per) * depth
            out[y, x, 0] = (byte >> sh) & ((1 << depth) - 1)
    return out


def _srgb_encode(v: np.ndarray) -> np.ndarray:
    # SRGB.decodeRGBAVecRaw -> applyGammaVec -> encodeRGBAVecRaw
    x = v.astype(np.float32) / np.float32(255.0)
    with np.errstate(divide="ignore"):
        g = np.where(x == 0, np.float32(0), np.where(x == 1, np.float32(1),
                     np.power(x.astype(np.float64), float(np.float32(1.0) / np.float32(2.2))).astype(np.float32)))
    return np.floor(np.float32(255.0) * g + np.float32(0.5)).astype(np.uint8)


def export_pixels(surface, profile=None) -> np.ndarray:
    """The pixel values z2d's exporter would write for this surface."""
    f = surface.format
    px = surface.pixels()
    if f == abi.FORMAT_RGBA:
        r, g, b, a = (px[..., i].astype(np.uint16) for i in range(4))
    elif f == abi.FORMAT_ARGB:
        b, g, r, a = (px[..., i].astype(np.uint16) for i in range(4))
    elif f == abi.FORMAT_RGB:
        r, g, b = (px[..., i].astype(np.uint16) for i in range(3))
        a = None
    elif f == abi.FORMAT_XRGB:
        b, g, r = (px[..., i].astype(np.uint16) for i in range(3))
        a = None
    else:
        return px[..., None].astype(np.uint8)
    if a is not None:  # pixel_vector.RGBA16.demultiply
        den = np.maximum(a, 1)
        r = np.where(a == 0, 0, r * 255 // den)
        g = np.where(a == 0, 0, g * 255 // den)
        b = np.where(a == 0, 0, b * 255 // den)
    chans = [r, g, b] + ([a] if a is not None else [])
    out = np.stack([c.astype(np.uint8) for c in chans], axis=-1)
    if profile == "srgb":
        out[..., :3] = _srgb_encode(out[..., :3])
    return out
