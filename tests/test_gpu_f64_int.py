"""The integer forms of f64 operations as compiled for the device give the
device's own f64 results (tests/f64_int_device_check.cu, built with nvcc
and run on the GPU; the host check is test_f64_int_check.py)."""
import os
import shutil
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_integer_forms_match_device_f64():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "f64_int_device_check")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "z2d_gb300", "csrc"),
                        os.path.join(HERE, "f64_int_device_check.cu"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "wrong 0" in r.stdout, r.stdout
