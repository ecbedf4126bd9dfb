"""Builds libz2dgpu.so (the C ABI of include/z2dgpu.h) for sm_103a, in-tree.

Each translation unit is compiled in parallel with nvcc, then linked into
z2d_gb300/_lib/libz2dgpu.so.  Flags that matter for parity:
  --fmad=false           no fused multiply-add (z2d's Zig code has none)
  --prec-div/--prec-sqrt IEEE division and square root (nvcc's default)
  -ffp-contract=off      the same for host-side descriptor arithmetic
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libz2dgpu.so"
SOURCES = ["capi.cu", "composite.cu", "composite_mask.cu", "composite_fused.cu", "composite_grad.cu", "fill.cu", "server.cu", "stroke.cpp", "stroke_gpu.cu", "hairline.cu", "png.cu", "tune.cu", "path_build.cu"]
HEADERS = ["z2d_pixel.cuh", "z2d_internal.h", "fill.cuh", "stroke.h", "stroke_geom.h", "stroke_gpu.cuh", "edges.cuh", "spline.cuh", "raster_px.cuh", "host_pool.h", "blue_noise_64x64.inc", "zig_math.cuh", "grad_fast.cuh", "zig_trig.cuh", "f64_int.cuh"]
ARCH = os.environ.get("Z2D_GPU_ARCH", "103a")


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libz2dgpu.so")
    return exe


# zlib compresses PNG exports when its header is installed (else stored blocks)
HAVE_ZLIB = any(pathlib.Path(d, "zlib.h").exists() for d in ("/usr/include", "/usr/local/include"))


def flags() -> list:
    return [
        f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-O3", "-lineinfo", "-std=c++17",
        "--fmad=false", "--prec-div=true", "--prec-sqrt=true",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
        f"-I{ROOT / 'include'}",
    ] + (["-DZ2D_HAVE_ZLIB"] if HAVE_ZLIB else [])


def _stale(target: pathlib.Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(pathlib.Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    OUT_DIR.mkdir(exist_ok=True)
    deps_common = [CSRC / h for h in HEADERS] + [ROOT / "include" / "z2dgpu.h", pathlib.Path(__file__)]
    objs = []
    jobs = []
    for src in SOURCES:
        obj = OUT_DIR / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + deps_common):
            cmd = [nvcc(), *flags(), "-c", str(CSRC / src), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode != 0:
                print(" ".join(cmd))
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        tmp = OUT_DIR / f"libz2dgpu.{os.getpid()}.so"
        cmd = [nvcc(), f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-shared", "-o", str(tmp),
               *[str(o) for o in objs], "-lcudart", "-ldl"] + (["-lz"] if HAVE_ZLIB else [])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout + r.stderr)
            raise RuntimeError("link of libz2dgpu.so failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
