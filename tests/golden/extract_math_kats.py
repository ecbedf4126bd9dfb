"""Extracts z2d's exact known answers for the Zig math the path calls into
math_kats.json.

Reads, as text, from the z2d tree:
  * src/color.zig, tests "SRGB.removeGamma" and "SRGB.applyGamma": the input
    colour and the expected channels, compared with expectEqualDeep, i.e.
    exact f32 values of std.math.pow(f32, x, 2.2) and pow(x, 1 / 2.2);
  * src/gradient.zig, test "Conic.getOffset": centre, start angle, optional
    scale matrix, pixel and the exact f32 offset (std.math.atan2(f64)).
The JSON is committed so the tests run where the z2d tree is absent.

Usage: python extract_math_kats.py <path to z2d>
"""
import json
import math
import pathlib
import re
import sys

FLOAT = r"-?\d+(?:\.\d+)?(?:e-?\d+)?"


def block(src: str, title: str) -> str:
    start = src.index(f'test "{title}"')
    end = src.index('\ntest "', start + 1)
    return src[start:end]


def gamma_cases(src: str, title: str, exponent: str):
    text = block(src, title)
    inp = re.search(rf"SRGB\.init\(({FLOAT}), ({FLOAT}), ({FLOAT}), ({FLOAT})\)", text)
    exp = re.search(rf"\.r = ({FLOAT}),\s*\.g = ({FLOAT}),\s*\.b = ({FLOAT}),", text)
    return [{"x": float(inp.group(i)), "exponent": exponent, "expected": float(exp.group(i))} for i in (1, 2, 3)]


def zig_const(expr: str) -> float:
    """The comptime expressions the conic cases use (math.pi / 4.0)."""
    expr = expr.strip()
    m = re.fullmatch(r"math\.pi / (\d+(?:\.\d+)?)", expr)
    if m:
        return math.pi / float(m.group(1))  # division by a power of two: exact
    return float(expr)


def conic_cases(src: str):
    text = block(src, "Conic.getOffset")
    out = []
    for m in re.finditer(r"\.\{\s*\.name = \"([^\"]+)\",(.*?)\n        \},", text, re.S):
        name, body = m.groups()
        f = dict(re.findall(r"\.(\w+) = ([^,\n]+),", body))
        scale = re.search(r"Transformation\.identity\.scale\(([\d.]+), ([\d.]+)\)", body)
        out.append({"name": name, "expected": float(f["expected"]), "center_x": zig_const(f["center_x"]),
                    "center_y": zig_const(f["center_y"]), "angle": zig_const(f["angle"]),
                    "scale": [float(scale.group(1)), float(scale.group(2))] if scale else None,
                    "x": int(f["x"]), "y": int(f["y"])})
    return out


def main() -> None:
    root = pathlib.Path(sys.argv[1])
    color = (root / "src" / "color.zig").read_text()
    gradient = (root / "src" / "gradient.zig").read_text()
    data = {"pow_f32": gamma_cases(color, "SRGB.removeGamma", "gamma") + gamma_cases(color, "SRGB.applyGamma",
                                                                                      "inverse_gamma"),
            "conic_offset": conic_cases(gradient)}
    out = pathlib.Path(__file__).with_name("math_kats.json")
    out.write_text(json.dumps(data, indent=1) + "\n")
    print({k: len(v) for k, v in data.items()})


if __name__ == "__main__":
    main()
