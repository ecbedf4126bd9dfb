"""The integer forms of f64 operations used by the flattener and the edge
builder (lerpHalf's a + (b - a) / 2, comparisons, scaling by a power of
two, rounding to an integer, conversion to f32) give the f64 results on
every operand they take (tests/f64_int_check.cu, built with nvcc as host
code and run on the CPU)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_integer_forms_match_f64():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "f64_int_check")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                        "-Xcompiler", "-ffp-contract=off",
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "z2d_gb300", "csrc"),
                        os.path.join(HERE, "f64_int_check.cu"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "wrong 0" in r.stdout, r.stdout
