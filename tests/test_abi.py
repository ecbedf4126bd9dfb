"""CPU checks of the C ABI boundary: the library builds for sm_103a, loads,
exports every symbol include/z2dgpu.h declares, and the ctypes mirror has
the header's struct layout.  No GPU call is made."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from z2d_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "z2dgpu.h")


def test_header_declares_exported_symbols():
    text = open(HEADER).read()
    declared = set(re.findall(r"Z2D_API\s+[\w\s\*]+?\b(z2dgpu_\w+)\s*\(", text))
    assert declared == set(abi.EXPORTED_SYMBOLS)


def test_library_loads_and_exports_every_symbol():
    from z2d_gb300 import native
    lib = native.load()
    for name in abi.EXPORTED_SYMBOLS:
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.z2dgpu_version()
    # pure host helper, no device needed
    assert lib.z2dgpu_surface_bytes(abi.FORMAT_ALPHA1, 3, 3) == 2
    assert lib.z2dgpu_surface_bytes(abi.FORMAT_RGBA, 3, 3) == 36


STRUCTS = ["z2d_pixel", "z2d_surface", "z2d_node", "z2d_color", "z2d_stop", "z2d_gradient", "z2d_pattern",
           "z2d_fill_opts", "z2d_param", "z2d_operation", "z2d_fill_cmd", "z2d_job", "z2d_stroke_opts",
           "z2d_draw_cmd"]


def test_ctypes_layout_matches_header():
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){"]
    for s in STRUCTS:
        src.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f, _ in getattr(abi, s)._fields_:
            src.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    src.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write("\n".join(src))
        subprocess.run(["gcc", "-o", exe, c], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    for s in STRUCTS:
        T = getattr(abi, s)
        assert int(got[s]) == C.sizeof(T), s
        for f, _ in T._fields_:
            assert int(got[f"{s}.{f}"]) == getattr(T, f).offset, f"{s}.{f}"
