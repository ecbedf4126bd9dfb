"""Extracts z2d's compositor known-answer tests into compositor_kats.json.

Reads the two table-driven tests "composite, all operators (integer)" and
"composite, all operators (float)" (src/compositor.zig:3078-3860 in z2d)
as text: each case gives an operator, background and foreground colors
(Color.InitArgs, turned into pixels with Pixel.fromColor) and the exact
RGBA result of compositor.runPixel.  The JSON is committed so the tests run
where the z2d tree is absent.

Usage: python extract_kats.py <path to z2d>/src/compositor.zig
"""
import json
import pathlib
import re
import sys

CASE = re.compile(
    r"\.operator = \.(\w+),\s*"
    r"\.expected = \.\{ \.rgba = \.\{ \.r = (\d+), \.g = (\d+), \.b = (\d+), \.a = (\d+) \} \},\s*"
    r"\.bg = \.\{ \.(rgba?) = \.\{ ([^}]*) \} \},\s*"
    r"\.fg = \.\{ \.(rgba?) = \.\{ ([^}]*) \} \},", re.S)


def block(src: str, title: str) -> str:
    start = src.index(f'test "{title}"')
    end = src.index('\ntest "', start + 1)
    return src[start:end]


def cases(text: str):
    out = []
    for m in CASE.finditer(text):
        op, r, g, b, a, bgk, bgv, fgk, fgv = m.groups()
        bg = [float(v) for v in bgv.split(",")]
        fg = [float(v) for v in fgv.split(",")]
        out.append({"op": op, "expected": [int(r), int(g), int(b), int(a)],
                    "bg": bg + [1.0] * (4 - len(bg)), "fg": fg + [1.0] * (4 - len(fg))})
    return out


def main() -> None:
    src = pathlib.Path(sys.argv[1]).read_text()
    data = {"integer": cases(block(src, "composite, all operators (integer)")),
            "float": cases(block(src, "composite, all operators (float)"))}
    out = pathlib.Path(__file__).with_name("compositor_kats.json")
    out.write_text(json.dumps(data, indent=1) + "\n")
    print({k: len(v) for k, v in data.items()})


if __name__ == "__main__":
    main()
