"""Writes blue_noise_64x64.inc: the 64x64 ordered-dither threshold table.

z2d's blue-noise dither (src/internal/blue_noise.zig:10, used by
src/Dither.zig:149-158 and src/internal/color_vector.zig:508-522) indexes a
4096-entry u16 table that z2d took from pixman (dither/blue-noise-64x64.h).
Bit-exact parity needs the very same numbers, so this script extracts them
from the z2d source tree and writes them as a C initializer list; the .inc is
committed so the GPU build (which has no access to the z2d tree) can include
it.  Usage:  python gen_blue_noise.py <path to z2d>/src/internal/blue_noise.zig
"""
import pathlib
import re
import sys


def main() -> None:
    src = pathlib.Path(sys.argv[1]).read_text()
    body = src[src.index("dither_blue_noise_64x64"):]
    body = body[body.index("{") + 1: body.index("}")]
    vals = [int(v) for v in re.findall(r"\d+", body)]
    if len(vals) != 4096:
        raise SystemExit(f"expected 4096 values, got {len(vals)}")
    out = pathlib.Path(__file__).with_name("blue_noise_64x64.inc")
    lines = ["/* 64x64 blue-noise dither thresholds (pixman dither/blue-noise-64x64.h,",
             " * as carried by z2d src/internal/blue_noise.zig).  Generated by",
             " * gen_blue_noise.py; index = (x mod 64) * 64 + (y mod 64). */"]
    for i in range(0, 4096, 16):
        lines.append(", ".join(str(v) for v in vals[i:i + 16]) + ",")
    out.write_text("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
