"""Benchmark: Mpix/s of z2d's fill+composite path on one GB300.

Workload (one "step"): the large plain-fill configuration -- a 4096x4096
RGBA surface holding seeded uniform premultiplied pixels, then 2,000 random
closed paths (3-64 segments, half lines / half cubic Beziers, control points
uniform in a random box of side 16-1024 px), fill rule alternating
even-odd / non-zero, random premultiplied pixel sources with alpha
U[32,255], src_over, drawn in order.  Synthetic, seeded.

Pixels counted (algorithmic, fixed before timing): the sum over fills of
the clamped multisample draw box (multisample.zig:46-78).

Arms of this implementation:
  value  -- batched: all 2,000 fills in one z2dgpu_fill_batch call on a
            device-resident surface (CUDA events on the library's stream).
  plain  -- the per-call drop-in: one z2dgpu_fill call per path, timed on the
            first 300 fills (reported beside).
  e2e    -- batched through the C ABI with a pinned HOST surface: the call
            uploads the surface and nodes and reads the surface back inside
            the timed region.
The surface (64 MiB) fits in L2, so L2 is flushed (256 MiB write) before
every timed step, outside the timed region.

--impl reference times the CPU restatement of z2d's path (z2d itself is Zig
and no Zig toolchain exists on these machines) on a bounded sample of the
same fills, single-threaded like z2d's painter.fill.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = H = 4096
N_FILLS = 2000
SEED = 2025
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
CPU_SAMPLE_FILLS = 2000   # cpu_baseline sample: the whole workload (~10-20 s single-threaded)
REF_STEP_FILLS = 400      # --impl reference: fills per timed step
PLAIN_FILLS = 300         # per-call arm: fills drawn with one z2dgpu_fill each
# Per-launch counters of the dominant kernels (DRAM bytes read + written,
# instructions executed), from ncu captures of this workload; the file
# records the hash of the CUDA sources of the build it captured, and the
# bench line says whether that is the build being measured.
COUNTERS_FILE = os.path.join(ROOT, "profiles", "counters_rgba4096_2000paths.json")


def source_hash():
    """SHA-256 (first 16 hex digits) of the library's CUDA and C++ sources:
    the identity of the build whose kernels are measured."""
    import hashlib
    csrc = os.path.join(ROOT, "z2d_gb300", "csrc")
    h = hashlib.sha256()
    for name in sorted(os.listdir(csrc)):
        if name.endswith((".cu", ".cuh", ".h", ".cpp", ".inc")):
            h.update(name.encode())
            with open(os.path.join(csrc, name), "rb") as f:
                h.update(f.read())
    with open(os.path.join(ROOT, "include", "z2dgpu.h"), "rb") as f:
        h.update(f.read())
    return h.hexdigest()[:16]


def load_counters():
    try:
        with open(COUNTERS_FILE) as f:
            return json.load(f)
    except Exception:
        return None


def kernel_counter(counters, kernel, key):
    """A captured per-launch counter, or None when it was not captured."""
    try:
        return counters["kernels"][kernel][key]
    except Exception:
        return None


NCU_KEYS = {"dram__bytes_read.sum": "dram_read", "dram__bytes_write.sum": "dram_write",
            "smsp__inst_executed.sum": "inst_executed", "gpu__time_duration.sum": "duration_ns"}


def write_counters(specs):
    """Writes the counters file from `ncu --csv` logs: each spec is
    NAME=CSV, NAME the key the bench reads (k_raster,
    k_mask_op_rgba_src_over_8192) and CSV one capture of that kernel
    (the last launch in it is taken; captures of one kernel with different
    metrics merge).  The file carries the source hash of
    the tree it was written from, which must be the tree that was
    captured."""
    import csv
    out = load_counters() or {}
    if out.get("source_hash") != source_hash():
        out = {}
    out["source_hash"] = source_hash()
    kernels = out.setdefault("kernels", {})
    for spec in specs:
        name, path = spec.split("=", 1)
        with open(path) as f:
            lines = f.read().splitlines()
        start = next(i for i, l in enumerate(lines) if l.startswith('"ID"'))
        launches = {}
        for row in csv.DictReader(lines[start:]):
            m = NCU_KEYS.get(row["Metric Name"])
            if m:
                d = launches.setdefault(row["ID"], {"kernel": row["Kernel Name"], "grid": row.get("Grid Size"),
                                                    "block": row.get("Block Size")})
                d[m] = float(row["Metric Value"].replace(",", ""))
        last = launches[max(launches, key=int)]
        k = kernels.setdefault(name, {})
        k.update(last)  # several captures of one kernel (metric groups) merge
        if "dram_read" in k and "dram_write" in k:
            k["dram_bytes"] = k["dram_read"] + k["dram_write"]
        k.setdefault("captures", []).append(os.path.basename(path))
    with open(COUNTERS_FILE, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out))


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


def settle_tuning(ctx, step, max_calls=12):
    """Runs `step` until the rasteriser's autotuner has decided the schedule
    for this kind of pass (it times one candidate schedule per pass at
    first); returns what it chose and how many passes that took."""
    calls = 0
    state = ctx.raster_tuning()
    while calls < max_calls:
        step()
        calls += 1
        state = ctx.raster_tuning()
        if state["decided"] != 0:
            break
    return dict(state, passes=calls)


def workload():
    from z2d_gb300.workloads import fill_box_pixels, premultiplied_background, random_fills
    rng = np.random.default_rng(SEED)
    bg = premultiplied_background(rng, W, H)
    fills = random_fills(SEED + 1, N_FILLS, W, H)
    px = [fill_box_pixels(n, W, H) for _, n, _ in fills]
    return bg, fills, px


def pack(fills):
    """One node array plus a ctypes command array (no per-call marshalling)."""
    import ctypes as C
    from z2d_gb300 import abi
    keep = []
    nodes = np.concatenate([n for _, n, _ in fills])
    cmds = (abi.z2d_fill_cmd * len(fills))()
    off = 0
    for i, (pat, n, opts) in enumerate(fills):
        p = pat.to_abi(keep)
        cmds[i].pattern = C.pointer(p)
        cmds[i].node_offset = off
        cmds[i].n_nodes = len(n)
        cmds[i].opts = opts.to_abi()
        off += len(n)
    return nodes, cmds, keep


class ClockSampler:
    def __init__(self, index=0):
        self.proc = None
        self.index = index
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"z2d_bench_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the timed region starts once samples are flowing
        t0 = time.time()
        while time.time() - t0 < 5 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.05)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def union_box_pixels(fills):
    """Pixels covered by the union of the fills' draw boxes (surface bytes
    the rasteriser must read and write at least once)."""
    import math
    from z2d_gb300 import abi
    cov = np.zeros((H, W), bool)
    for _, nodes, _ in fills:
        pts = []
        for nd in nodes:
            t = nd["tag"]
            if t in (abi.MOVE_TO, abi.LINE_TO):
                pts.append(nd["p"][:2])
            elif t == abi.CURVE_TO:
                pts.extend([nd["p"][0:2], nd["p"][2:4], nd["p"][4:6]])
        p = np.array(pts)
        x0 = min(max(int(math.floor(p[:, 0].min())), 0), W - 1)
        x1 = min(max(int(math.ceil(p[:, 0].max())), x0), W)
        y0 = min(max(int(math.floor(p[:, 1].min())), 0), H - 1)
        y1 = min(max(int(math.ceil(p[:, 1].max())), y0), H - 1)
        cov[y0:y1 + 1, x0:x1] = True
    return int(cov.sum())


def cpu_sample(bg, fills, px, n_fills, snapshot_at=None):
    """The oracle on the whole workload, single-threaded: Mpix/s, seconds,
    the final surface and a copy of the surface after `snapshot_at` fills
    (both kept for the parity check of the GPU arms)."""
    from oracle import Oracle
    from z2d_gb300.surface import Surface
    o = Oracle()
    s = Surface("rgba", W, H, bg.copy())
    snap = None
    dt = 0.0
    for i, (pat, nodes, opts) in enumerate(fills[:n_fills]):
        if i == snapshot_at:
            snap = s.data.copy()
        t0 = time.perf_counter()
        o.fill(s, pat, nodes, opts)
        dt += time.perf_counter() - t0
    if snapshot_at is not None and snapshot_at >= n_fills:
        snap = s.data.copy()
    return sum(px[:n_fills]) / 1e6 / dt, dt, s.data, snap


def diff_stats(got, ref):
    """Differing bytes, differing pixels and the largest channel difference
    of two RGBA surfaces."""
    a = np.asarray(got, np.uint8).reshape(-1, 4).astype(np.int16)
    b = np.asarray(ref, np.uint8).reshape(-1, 4).astype(np.int16)
    d = np.abs(a - b)
    return {"differing_bytes": int((d > 0).sum()), "differing_pixels": int((d > 0).any(1).sum()),
            "max_diff": int(d.max(initial=0))}


def issue_roofline(counters, launch_ms, clk):
    """k_raster is bound by instruction issue, not HBM: instructions
    executed per launch (ncu, smsp__inst_executed.sum) over its measured
    duration, against the issue peak of one warp instruction per cycle per
    SM sub-partition (4 per SM) at the SM clock sampled during the run."""
    inst = kernel_counter(counters, "k_raster", "inst_executed")
    if not inst or not launch_ms:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6  # warp instructions per second
    achieved = inst / (launch_ms / 1e3)
    return {"bound": "issue", "kernel": "k_raster", "achieved": achieved, "peak": peak,
            "unit": "warp inst/s", "frac": achieved / peak, "inst_per_launch": inst,
            "source": os.path.relpath(COUNTERS_FILE, ROOT), "sm_mhz": mhz,
            "note": "peak = SMs x 4 sub-partitions x 1 warp instruction per cycle x the sampled SM clock"}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_threads_step(lib, surfaces, args_list, n_threads):
    """One reference step: every thread draws the sample fills, in order, on
    its own copy of the surface (z2d's painter.fill is sequential per
    surface, so independent surfaces are how it uses more cores).  The
    ctypes call releases the GIL while the C++ fill runs."""
    from concurrent.futures import ThreadPoolExecutor

    def work(i):
        s = surfaces[i]
        for pat, nodes, n, opts in args_list:
            lib.z2doracle_fill(s, pat, nodes, n, opts)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(n_threads) as ex:
        list(ex.map(work, range(n_threads)))
    return time.perf_counter() - t0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import ctypes as C
    from oracle import build_oracle, load_oracle
    from z2d_gb300 import abi
    from z2d_gb300.types import nodes_to_abi
    bg, fills, px = workload()
    build_oracle()
    lib = load_oracle()
    n_threads = host_threads()
    keep = []
    args_list = []
    for pat, nodes, opts in fills[:REF_STEP_FILLS]:
        p = pat.to_abi(keep)
        o = opts.to_abi()
        arr = nodes_to_abi(nodes)
        keep += [p, o, arr]
        args_list.append((C.byref(p), arr, len(nodes), C.byref(o)))
    hosts = [bg.copy() for _ in range(n_threads)]
    surfaces = []
    for h in hosts:
        sfc = abi.z2d_surface(format=abi.FORMAT_RGBA, width=W, height=H, location=abi.MEM_HOST,
                              data=h.ctypes.data_as(C.c_void_p))
        keep.append(sfc)
        surfaces.append(C.byref(sfc))
    for _ in range(args.warmup):
        cpu_threads_step(lib, surfaces, args_list[:8], n_threads)
    times = []
    for _ in range(args.steps):
        for h in hosts:
            h[:] = bg
        times.append(cpu_threads_step(lib, surfaces, args_list, n_threads))
    mpix_step = n_threads * sum(px[:REF_STEP_FILLS]) / 1e6
    value = mpix_step * args.steps / sum(times)
    sample = (f"first {REF_STEP_FILLS} of the {N_FILLS} fills of the 4096x4096 workload per step, "
              f"on {n_threads} independent surface copies (one per host thread)")
    line = {
        "impl": "reference", "metric": "Mpix/s fill+composite (src_over, 4096x4096 RGBA, 2000 random paths)",
        "value": value, "unit": "Mpix/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded)",
        "config": {"workload": "plain_large_4096x4096_2000_paths", "surface": "rgba 4096x4096", "paths": N_FILLS},
        "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": n_threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "z2d is Zig and no Zig toolchain exists here, so the C++ restatement of its fill path "
                "is timed on all host threads, one surface per thread",
    }
    print(json.dumps(line))


def compositor_sweep(ctx, stream, dev, reps=3):
    """The compositor configuration on one surface: 8192x8192 RGBA
    destination with seeded premultiplied pixels, a seeded alpha8 mask, and
    the batch [dst_in(dst = pixel source, src = mask), op] for every integer
    operator.  HBM bound: 4 B read + 4 B written + 1 B mask per pixel.  The
    surfaces (288 MiB) exceed L2, so no flush is needed."""
    import torch
    from z2d_gb300 import abi, compositor
    from z2d_gb300.surface import Surface
    from z2d_gb300.types import Operation, Pattern, Pixel
    n = 8192
    g = torch.Generator(device=dev)
    g.manual_seed(SEED)
    a = torch.randint(0, 256, (n * n,), device=dev, generator=g, dtype=torch.int32)
    rgb = torch.randint(0, 256, (n * n, 3), device=dev, generator=g, dtype=torch.int32) * (a[:, None] + 1) // 256
    dst_t = torch.cat([rgb, a[:, None]], 1).to(torch.uint8).reshape(-1).contiguous()
    base = dst_t.clone()
    mask_t = torch.randint(0, 256, (n * n,), device=dev, generator=g, dtype=torch.int32).to(torch.uint8)
    dst = Surface("rgba", n, n, dst_t)
    mask = Surface("alpha8", n, n, mask_t)
    src = Pattern.from_pixel(Pixel.rgba(90, 40, 160, 200))
    int_ops = [o for o in abi.OPERATORS if o not in abi.FLOAT_ONLY_OPS]
    per_op = {}
    for op in int_ops:
        ops = [Operation("dst_in", dst=src, src=mask), Operation(op)]
        compositor.SurfaceCompositor.run(dst, 0, 0, ops, ctx=ctx)  # warm
        ctx.set_timing(True)
        for _ in range(reps):
            compositor.SurfaceCompositor.run(dst, 0, 0, ops, ctx=ctx)
        ms, nl = ctx.kernel_ms("composite")
        ctx.set_timing(False)
        per_op[op] = ms / max(nl, 1)
        with torch.cuda.stream(stream):
            dst_t.copy_(base)
    stream.synchronize()
    bytes_px = 4 + 4 + 1
    px = n * n
    so = per_op["src_over"]
    mean_ms = sum(per_op.values()) / len(per_op)
    return {
        "workload": "8192x8192 rgba, alpha8 mask, [dst_in(pixel, mask), op], 21 integer operators",
        "mpix_per_s_src_over": px / 1e6 / (so / 1e3),
        "gbs_src_over": bytes_px * px / (so / 1e3) / 1e9,
        "gbs_mean_all_ops": bytes_px * px / (mean_ms / 1e3) / 1e9,
        "ms_per_launch": {k: round(v, 4) for k, v in per_op.items()},
        "bytes_per_px": bytes_px,
    }


def compositor_breadth(ctx, stream, dev, reps=2):
    """The rest of the compositor configuration, one timed pass each on
    8192x8192 surfaces with the same [dst_in(dst = source, src = mask), op]
    batch: the other pixel formats (integer operators, pixel source), the
    float operators on RGBA, and gradient / dither sources (linear, radial,
    conic x linear_rgb, srgb, hsl x no dither, Bayer, blue noise; 4 stops)."""
    import torch
    from z2d_gb300 import abi, compositor
    from z2d_gb300.surface import Surface
    from z2d_gb300.types import Color, Gradient, Operation, Pattern, Pixel
    n = BREADTH_SIZE
    k = n / 8192  # geometry of the gradients scales with the surface
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 7)
    mask = Surface("alpha8", n, n, torch.randint(0, 256, (n * n,), device=dev, generator=g,
                                                  dtype=torch.int32).to(torch.uint8))
    pix = Pattern.from_pixel(Pixel.rgba(90, 40, 160, 200))

    def timed(dst, src, op, precision="integer"):
        ops = [Operation("dst_in", dst=src, src=mask), Operation(op)]
        compositor.SurfaceCompositor.run(dst, 0, 0, ops, precision, ctx=ctx)
        ctx.set_timing(True)
        for _ in range(reps):
            compositor.SurfaceCompositor.run(dst, 0, 0, ops, precision, ctx=ctx)
        ms, nl = ctx.kernel_ms("composite")
        ctx.set_timing(False)
        return ms / max(nl, 1)

    out = {"formats": {}, "float_ops_rgba": {}, "sources_rgba_src_over": {}}
    bpp = {"rgb": 4, "alpha8": 1, "alpha4": 0.5, "alpha2": 0.25, "alpha1": 0.125}
    for fmt, b in bpp.items():
        if BREADTH_ONLY and BREADTH_ONLY not in fmt:
            continue
        nbytes = abi.surface_bytes(abi.FORMAT_NAMES.index(fmt), n, n)
        t = torch.randint(0, 256, ((nbytes + 3) // 4 * 4,), device=dev, generator=g, dtype=torch.int32).to(torch.uint8)
        dst = Surface(fmt, n, n, t)
        res = {}
        for op in ("src_over", "xor", "multiply"):
            ms = timed(dst, pix, op)
            res[op] = {"ms": round(ms, 4), "gbs": (2 * b + 1) * n * n / (ms / 1e3) / 1e9}
        out["formats"][fmt] = res
        del dst, t
    t = torch.randint(0, 256, (n * n * 4,), device=dev, generator=g, dtype=torch.int32).to(torch.uint8)
    dst = Surface("rgba", n, n, t)
    for op in ["src_over"] + sorted(abi.FLOAT_ONLY_OPS):
        if BREADTH_ONLY and BREADTH_ONLY not in "float/" + op:
            continue
        ms = timed(dst, pix, op, "float")
        out["float_ops_rgba"][op] = {"ms": round(ms, 4), "mpix_s": n * n / 1e6 / (ms / 1e3)}
    for kind in ("linear", "radial", "conic"):
        for method in ("linear_rgb", "srgb", "hsl"):
            gr = {"linear": Gradient.linear(100 * k, 200 * k, 8000 * k, 7000 * k, method=method),
                  "radial": Gradient.radial(4000 * k, 4000 * k, 50 * k, 4100 * k, 4200 * k, 5000 * k, method=method),
                  "conic": Gradient.conic(4096 * k, 4096 * k, 0.3, method=method)}[kind]
            for i, c in enumerate((Color.rgb(1, 0, 0, 1), Color.rgb(0, 1, 0, 0.6), Color.rgb(0, 0, 1, 0.8),
                                   Color.rgb(1, 1, 0, 1))):
                gr.add_stop(i / 3, c)
            for dither in ("none", "bayer", "blue_noise"):
                if BREADTH_ONLY and BREADTH_ONLY not in f"{kind}/{method}/{dither}":
                    continue
                src = Pattern.from_gradient(gr) if dither == "none" else Pattern.dither(dither, gr, 8)
                ms = timed(dst, src, "src_over")
                out["sources_rgba_src_over"][f"{kind}/{method}/{dither}"] = {
                    "ms": round(ms, 4), "mpix_s": n * n / 1e6 / (ms / 1e3)}
    stream.synchronize()
    return out


BREADTH_SIZE = 8192       # compositor breadth arm: side of its surfaces
BREADTH_ONLY = ""         # ... and only the cells whose name contains this (profiling captures)
N_JOBS = 4096             # batched-jobs arm: RGBA jobs, sides log-uniform [16, 2048], 1-200 paths each
JOBS_PLAIN_FILLS = 1500   # per-call sample of the jobs arm (complete jobs, in order)


JOBS_STROKED = 0.3        # share of paths stroked instead of filled
JOBS_SURFACE_SAMPLE = 512  # per-surface arm: the first jobs, one z2dgpu_draw_jobs call each


def jobs_arm(ctx, stream, dev, steps=3):
    """The batched-jobs configuration: N_JOBS independent RGBA surfaces, each
    with its own ordered paths (z2d_gb300.workloads.batched_jobs); 30 % of
    the paths are stroked (width U[0.5, 20], join and cap uniform, half of
    them dashed with 2-6 dash lengths in [1, 40]), the rest filled; one
    z2dgpu_draw_jobs call per step.  Pixels counted: the sum of the job
    surfaces' w x h.  Beside it: one call per surface on the first jobs, one
    painter call per path on the first jobs, and the CPU restatement on all
    host threads (one job per thread) on a sample."""
    import torch
    from z2d_gb300 import abi, painter
    from z2d_gb300.batch import PackedDrawBatch
    from z2d_gb300.surface import Surface
    from z2d_gb300.types import StrokeOptions
    from z2d_gb300.workloads import batched_jobs, job_fills
    t_gen = time.perf_counter()
    jobs = batched_jobs(SEED + 11, N_JOBS)
    srng = np.random.default_rng(SEED + 13)
    nodes, offs, cnts, pxs, rules, cmd_off, cmd_cnt = [], [], [], [], [], [], []
    base = ncmd = 0
    for w, h, nd, off, cnt, px, rl in jobs:
        nodes.append(nd)
        offs.append(off + base)
        cnts.append(cnt)
        pxs.append(px)
        rules.append(rl)
        cmd_off.append(ncmd)
        cmd_cnt.append(len(off))
        base += len(nd)
        ncmd += len(off)
    stroke = srng.random(ncmd) < JOBS_STROKED
    widths = srng.uniform(0.5, 20.0, ncmd)
    joins = srng.integers(0, 3, ncmd)
    caps = srng.integers(0, 3, ncmd)
    dashed = stroke & (srng.random(ncmd) < 0.5)
    dashes = [tuple(srng.uniform(1.0, 40.0, int(srng.integers(2, 7)))) if d else () for d in dashed]
    pb = PackedDrawBatch(np.concatenate(nodes), np.concatenate(offs), np.concatenate(cnts), np.concatenate(pxs),
                         np.concatenate(rules), stroke, widths, joins, caps, dashes)
    t_gen = time.perf_counter() - t_gen
    sizes = [w * h * 4 for w, h, *_ in jobs]
    starts = []
    tot = 0
    for sz in sizes:
        starts.append(tot)
        tot += (sz + 255) // 256 * 256
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 12)
    a = torch.randint(0, 256, (tot // 4,), device=dev, generator=g, dtype=torch.int32)
    rgb = torch.randint(0, 256, (tot // 4, 3), device=dev, generator=g, dtype=torch.int32) * (a[:, None] + 1) // 256
    pristine = torch.cat([rgb, a[:, None]], 1).to(torch.uint8).reshape(-1).contiguous()
    del a, rgb
    buf = pristine.clone()
    surfaces = [Surface("rgba", w, h, buf[o:o + sz]) for (w, h, *_), o, sz in zip(jobs, starts, sizes)]
    pb.set_jobs(surfaces, cmd_off, cmd_cnt)
    mpix = sum(w * h for w, h, *_ in jobs) / 1e6

    def restore():
        with torch.cuda.stream(stream):
            buf.copy_(pristine)
        stream.synchronize()

    restore()
    pb.draw_jobs(ctx)  # warm

    def tune_step():
        restore()
        pb.draw_jobs(ctx)
        stream.synchronize()

    tuning = settle_tuning(ctx, tune_step)
    ctx.set_timing(True)
    walls = []
    for _ in range(steps):
        restore()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push("jobs_step")  # lets a profiler select these launches
        pb.draw_jobs(ctx)
        stream.synchronize()
        torch.cuda.nvtx.range_pop()
        walls.append(time.perf_counter() - t0)
    stage_ms = {k: ctx.kernel_ms(k)[0] / steps for k in ("flatten", "stroke", "bins", "raster")}
    out_jobs = buf.cpu().numpy()  # the last timed pass's surfaces, for the parity check
    pristine_host = pristine.cpu().numpy()
    ctx.set_timing(False)
    # one call per surface, first jobs
    restore()
    ns = min(JOBS_SURFACE_SAMPLE, len(jobs))
    t0 = time.perf_counter()
    for j in range(ns):
        pb.draw_job(j, ctx)
    stream.synchronize()
    per_surface_s = time.perf_counter() - t0
    per_surface_mpix = sum(jobs[j][0] * jobs[j][1] for j in range(ns)) / 1e6
    # one painter call per path on whole jobs from the start
    restore()

    def ops_of(j):
        out = []
        for k, (pat, nd, fo) in enumerate(job_fills(jobs[j])):
            i = cmd_off[j] + k
            if stroke[i]:
                so = StrokeOptions(line_width=float(widths[i]), line_join=("miter", "round", "bevel")[joins[i]],
                                   line_cap=("butt", "round", "square")[caps[i]], dashes=dashes[i])
                out.append(("stroke", pat, nd, so))
            else:
                out.append(("fill", pat, nd, fo))
        return out

    k, nf = 0, 0
    while k < len(jobs) and nf < JOBS_PLAIN_FILLS:
        nf += cmd_cnt[k]
        k += 1
    plain_ops = [(surfaces[j], ops_of(j)) for j in range(k)]
    t0 = time.perf_counter()
    for sfc, ops in plain_ops:
        for kind, pat, nd, o in ops:
            (painter.fill if kind == "fill" else painter.stroke)(sfc, pat, nd, o, ctx=ctx)
    stream.synchronize()
    plain_s = time.perf_counter() - t0
    plain_mpix = sum(jobs[j][0] * jobs[j][1] for j in range(k)) / 1e6
    out = {
        "workload": f"{N_JOBS} RGBA jobs, sides log-uniform [16, 2048], 1-200 paths each, "
                    f"{int(JOBS_STROKED * 100)}% stroked (half of those dashed)",
        "jobs": N_JOBS, "commands": int(ncmd), "strokes": int(stroke.sum()), "nodes": int(base),
        "mpix_per_step": mpix,
        "value": mpix * steps / sum(walls), "unit": "Mpix/s (sum of job surfaces w x h)",
        "ms_per_step": 1000 * sum(walls) / steps,
        "stage_ms_per_step": stage_ms,
        "per_surface": {"value": per_surface_mpix / per_surface_s, "calls": ns},
        "plain": {"value": plain_mpix / plain_s, "jobs": k, "calls": nf},
        "note": "wall time of the call (host validation, stroke building, packing, uploads, kernels); "
                "inputs in host memory, surfaces on the device",
        "generation_s": t_gen,
        "autotune": tuning,
    }
    del buf, pristine, surfaces
    # CPU restatement on all host threads, one job per thread: every job,
    # drawn from its seeded background, is compared with the GPU's pass
    from oracle import Oracle, load_oracle
    from concurrent.futures import ThreadPoolExecutor
    import ctypes as C
    from z2d_gb300 import abi as A
    from z2d_gb300.types import nodes_to_abi
    lib = load_oracle()
    orc = Oracle()

    def prepare(j):
        w, h = jobs[j][0], jobs[j][1]
        host = pristine_host[starts[j]:starts[j] + sizes[j]].copy()
        keep, calls = [], []
        for kind, pat, nd, o in ops_of(j):
            p = pat.to_abi(keep)
            keep.append(p)
            if kind == "fill":
                fo, arr = o.to_abi(), nodes_to_abi(nd)
                keep += [fo, arr]
                calls.append(("fill", C.byref(p), arr, len(nd), C.byref(fo)))
            else:
                contours, _ = orc.stroke_contours(nd, o, "rgba")
                pts = np.ascontiguousarray(np.concatenate(contours) if contours else np.zeros((1, 2)))
                ends = (np.cumsum([len(c_) for c_ in contours]) if contours else np.zeros(1)).astype(np.uint64)
                fo = A.z2d_fill_opts(anti_aliasing=A.AA_DEFAULT, fill_rule=A.FILL_NON_ZERO, op=A.OP["src_over"],
                                     precision=A.PRECISION_INTEGER, tolerance=0.1)
                keep += [pts, ends, fo]
                calls.append(("stroke", C.byref(p), pts, ends, len(contours), C.byref(fo)))
        sfc = A.z2d_surface(format=A.FORMAT_RGBA, width=w, height=h, location=A.MEM_HOST,
                            data=host.ctypes.data_as(C.c_void_p))
        return (sfc, host, keep, calls)

    def run(item):
        sfc, _, _, calls = item
        for c_ in calls:
            if c_[0] == "fill":
                lib.z2doracle_fill(C.byref(sfc), c_[1], c_[2], c_[3], c_[4])
            else:
                lib.z2doracle_fill_contours(C.byref(sfc), c_[1], c_[2].ctypes.data_as(C.POINTER(C.c_double)),
                                            c_[3].ctypes.data_as(C.POINTER(C.c_uint64)), c_[4], c_[5])

    nt = host_threads()
    k = nf = 0
    cpu_s = 0.0
    bad_jobs, bad_px = [], 0
    with ThreadPoolExecutor(nt) as ex:
        while k < len(jobs):
            chunk = list(range(k, min(len(jobs), k + 4 * nt)))
            work = [prepare(j) for j in chunk]
            t0 = time.perf_counter()
            list(ex.map(run, work))
            cpu_s += time.perf_counter() - t0
            for j, item in zip(chunk, work):
                got = out_jobs[starts[j]:starts[j] + sizes[j]]
                if not np.array_equal(got, item[1]):
                    bad_jobs.append(j)
                    bad_px += int((got.reshape(-1, 4) != item[1].reshape(-1, 4)).any(1).sum())
            k = chunk[-1] + 1
            nf += sum(cmd_cnt[j] for j in chunk)
    out["cpu"] = {"value": sum(jobs[j][0] * jobs[j][1] for j in range(k)) / 1e6 / cpu_s, "jobs": k, "commands": nf,
                  "cores": nt, "seconds": cpu_s, "kind": "port",
                  "note": "every job; stroke polygons built beforehand by the oracle's stroker (not timed), fills "
                          "and polygons rasterised"}
    out["parity"] = {"jobs_checked": k, "differing_jobs": len(bad_jobs), "differing_pixels": bad_px,
                     "first_differing": bad_jobs[:8],
                     "reference": "oracle on host threads, every job from its seeded background; strokes "
                                  "tessellated by the oracle's own stroker"}
    return out


SERVE_RATES = (5000, 20000, 50000)  # requests per second (Poisson arrivals)
SERVE_SECONDS = 1.5                 # arrival window per rate


def png_arm(ctx, surf, peak_gbs):
    """PNG export of the benchmark's 4096x4096 RGBA surface (device
    resident, as the batched arm leaves it): the exporter's encoding kernel
    k_png_rows (4 B read and 4 B written per pixel, plus a filter byte per
    row) timed with CUDA events (the context's "export" stage), and the
    whole file: device encoding, copy back and zlib on the host."""
    from z2d_gb300 import png
    import torch
    reps = 5
    png.scanlines(surf, None, ctx)  # warm
    ctx.set_timing(True)
    for _ in range(reps):
        torch.cuda.nvtx.range_push("png_export")
        png.scanlines(surf, None, ctx)
        torch.cuda.nvtx.range_pop()
    ms = ctx.kernel_ms("export")[0] / reps
    ctx.set_timing(False)
    t0 = time.perf_counter()
    data = png.encode(surf, None, ctx)
    file_s = time.perf_counter() - t0
    alg = W * H * 4 + H * (1 + 4 * W)
    gbs = alg / (ms / 1e3) / 1e9
    return {"kernel": "k_png_rows", "kernel_ms": ms, "alg_bytes": alg, "gbs": gbs, "frac_of_measured_hbm": gbs / peak_gbs,
            "file_ms": file_s * 1e3, "png_bytes": len(data), "file_mpix_s": W * H / 1e6 / file_s,
            "note": "file = device encoding + copy back + zlib default level on one host thread"}


SERVE_LANES = 3           # server lanes (batches drawn concurrently)
SERVE_WAIT_US = 0         # batching window: none, a free lane takes what is queued
SERVE_POOL = 4 << 30      # device surface pool of the server
SERVE_OUT_RING = 2048     # host result buffers, reused round-robin by the requests
SERVE_PARITY = 4096       # requests of the fastest rate compared with the oracle


def serving_arm(dev):
    """The serving configuration: requests arrive as a Poisson process and go
    through the continuous-batching server (z2d_gb300.server: SERVE_LANES
    lanes drawing batches concurrently, up to 512 requests per batch; a free
    lane takes whatever is queued, so batches grow with the load).  Each request draws on a surface the server
    allocates from its device pool (cleared) and reads the result back into
    a host buffer, so latency is end to end (submit to pixels in host
    memory).  Mix: 80 % glyph-like requests (one outline of 20-200 cubics on
    a 64x64 RGBA surface; half with a linear-gradient source), 20 % jobs of
    the batched-jobs distribution with sides up to 512.  Reported per rate:
    achieved request rate, latency p50/p99 (measured by the server) and
    Mpix/s of surface area.  The last SERVE_PARITY requests of the fastest
    rate are compared with the same requests drawn alone by the oracle."""
    import ctypes as C
    import threading
    from z2d_gb300 import abi
    from z2d_gb300.server import Server
    from z2d_gb300.types import Color, FillOptions, Gradient, Pattern
    from z2d_gb300.workloads import batched_jobs, glyph_path, job_fills, random_premultiplied_pixel
    rng = np.random.default_rng(SEED + 21)
    n_req = int(max(SERVE_RATES) * SERVE_SECONDS)
    pool = 2000  # distinct request contents; request k draws pool entry k % pool
    jobs = batched_jobs(SEED + 22, pool // 5, side_lo=16, side_hi=512, paths_lo=1, paths_hi=50)
    grad = Gradient.linear(0, 0, 64, 64)
    grad.add_stop(0.0, Color.rgb(0.9, 0.1, 0.1, 1.0))
    grad.add_stop(1.0, Color.rgb(0.1, 0.2, 0.9, 0.8))
    reqs = []  # (w, h, nodes, cmds ctypes array, keep, fills)
    ji = 0
    for i in range(pool):
        if i % 5 == 4 and ji < len(jobs):
            w, h = jobs[ji][0], jobs[ji][1]
            fills = job_fills(jobs[ji])
            ji += 1
        else:
            w = h = 64
            pat = Pattern.from_gradient(grad) if i % 2 else Pattern.from_pixel(random_premultiplied_pixel(rng))
            fills = [(pat, glyph_path(rng), FillOptions())]
        keep = []
        cmds = (abi.z2d_fill_cmd * len(fills))()
        arrs, off = [], 0
        for k, (pat, nd, opts) in enumerate(fills):
            p = pat.to_abi(keep)
            keep.append(p)
            cmds[k].pattern = C.pointer(p)
            cmds[k].node_offset = off
            cmds[k].n_nodes = len(nd)
            cmds[k].opts = opts.to_abi()
            off += len(nd)
            arrs.append(nd)
        reqs.append((w, h, np.ascontiguousarray(np.concatenate(arrs)), cmds, keep, fills))
    # request k reads back into ring slot k % SERVE_OUT_RING (one slot holds
    # the largest surface, 512x512 RGBA); at the fastest rate the ring spans
    # ~40 ms of arrivals, far beyond a request's latency, so no two requests
    # in flight share a slot
    ring = np.zeros((SERVE_OUT_RING, 512 * 512 * 4), np.uint8)
    results = {}
    parity = None
    with Server(max_batch_jobs=512, max_wait_us=SERVE_WAIT_US, lanes=SERVE_LANES, pool_bytes=SERVE_POOL) as srv:
        lib = srv.lib

        def out_buf(k):
            w, h = reqs[k % pool][0], reqs[k % pool][1]
            return ring[k % SERVE_OUT_RING, :w * h * 4]

        # warm-up: a burst of every request content, so that the lanes' device
        # buffers have grown to their working size before anything is timed
        # (growing one synchronises the device)
        for rep in range(2):
            ts = [_submit_new(lib, srv.handle, reqs[i][0], reqs[i][1], out_buf(i), reqs[i][2], reqs[i][3])
                  for i in range(pool)]
            for t in ts:
                srv.wait(t)
        for rate in SERVE_RATES:
            n = int(rate * SERVE_SECONDS)
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
            bufs = [out_buf(k) for k in range(n)]
            tickets = [0] * n
            lat = [0.0] * n
            submitted = threading.Semaphore(0)
            check_from = n - SERVE_PARITY if rate == max(SERVE_RATES) else n
            kept = []

            def waiter():
                for k in range(n):
                    submitted.acquire()
                    lat[k] = srv.wait(tickets[k])
                    if k >= check_from:  # copied before its ring slot is reused
                        kept.append((k, bufs[k].copy()))

            th = threading.Thread(target=waiter)
            th.start()
            t0 = time.perf_counter()
            for k in range(n):
                while time.perf_counter() - t0 < arrivals[k]:
                    pass
                w, h, nodes, cmds, _, _ = reqs[k % pool]
                tickets[k] = _submit_new(lib, srv.handle, w, h, bufs[k], nodes, cmds)
                submitted.release()
            t_sub = time.perf_counter() - t0
            th.join()
            wall = time.perf_counter() - t0
            ls = sorted(lat)
            px = sum(reqs[k % pool][0] * reqs[k % pool][1] for k in range(n))
            results[str(rate)] = {"requests": n, "offered_per_s": rate, "submitted_per_s": n / t_sub,
                                  "completed_per_s": n / wall, "p50_us": ls[n // 2], "p99_us": ls[int(n * 0.99) - 1],
                                  "mpix_s": px / 1e6 / wall}
            if kept:
                parity = {"rate": rate, "requests_checked": len(kept), "kept": kept}
        info = srv.info()
    if parity is not None:
        from oracle import Oracle
        from z2d_gb300.surface import Surface
        o = Oracle()
        bad = 0
        for k, got in parity.pop("kept"):
            w, h, _, _, _, fills = reqs[k % pool]
            ref = Surface.init("rgba", w, h)
            for pat, nd, opts in fills:
                o.fill(ref, pat, nd, opts)
            bad += int(not np.array_equal(got, ref.data))
        parity["differing_requests"] = bad
        parity["reference"] = "each request drawn alone on a cleared surface by the oracle"
    return {"workload": "Poisson arrivals; 80% glyphs (20-200 cubics, 64x64, half gradient), 20% jobs "
                        "(sides 16-512, 1-50 paths); one pool surface per request, result read back to host",
            "server": {"max_batch_jobs": 512, "max_wait_us": SERVE_WAIT_US, "lanes": SERVE_LANES, "pool_bytes": SERVE_POOL,
                       "info": info},
            "rates": results, "parity": parity}


def _submit_new(lib, handle, w, h, out, nodes, cmds):
    import ctypes as C
    from z2d_gb300 import abi
    from z2d_gb300.native import check
    t = C.c_uint64()
    check(lib.z2dgpu_server_submit_new(handle, abi.FORMAT_RGBA, w, h, None, out.ctypes.data_as(C.c_void_p),
                                       nodes.ctypes.data_as(C.POINTER(abi.z2d_node)), len(nodes), cmds, len(cmds),
                                       C.byref(t)))
    return t.value


def star_latency(ctx, dev, iters=200):
    """The small plain configuration: the 300x300 star, one painter.fill per
    call, on a device surface and on a host surface (synchronous calls:
    host wall time per call, p50/p99)."""
    import torch
    from z2d_gb300 import painter
    from z2d_gb300.surface import Surface
    from z2d_gb300.workloads import fill_box_pixels, star_300
    w, h, nodes, pat, opts = star_300()
    px = fill_box_pixels(nodes, w, h)
    res = {}
    for where in ("device", "host"):
        s = Surface.init("rgba", w, h)
        if where == "device":
            s = s.to_device(dev)
        lat = []
        for i in range(iters + 5):
            t0 = time.perf_counter()
            painter.fill(s, pat, nodes, opts, ctx=ctx)
            if where == "device":
                ctx.synchronize()
            if i >= 5:
                lat.append((time.perf_counter() - t0) * 1e6)
        lat.sort()
        res[where] = {"p50_us": lat[len(lat) // 2], "p99_us": lat[int(len(lat) * 0.99) - 1],
                      "mpix_s": px / 1e6 / (statistics.mean(lat) / 1e6)}
    res["fill_box_px"] = px
    return res


def max_over_ranks(ms, world, device):
    """The slowest rank's time: every rank runs the same replica of the
    workload, so the job's time is the maximum (an all-reduce of one value;
    no data moves between ranks otherwise)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(world, mpix_step, steps, total_ms):
    """Whole-job throughput of `world` replicas (weak scaling): every rank
    drew mpix_step per step for `steps` steps in at most total_ms."""
    return world * mpix_step * steps / (total_ms / 1e3)


def run_ours(args):
    import torch
    import torch.distributed as dist
    from z2d_gb300 import painter
    from z2d_gb300.native import Context
    from z2d_gb300.surface import Surface

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    bg, fills, px = workload()
    mpix_step = sum(px) / 1e6
    nodes, cmds, keep = pack(fills)

    stream = torch.cuda.Stream(device=dev)
    ctx = Context(local, stream)
    bg_dev = torch.from_numpy(bg).to(dev)
    surf_t = bg_dev.clone()
    surf = Surface("rgba", W, H, surf_t)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def restore():
        with torch.cuda.stream(stream):
            surf_t.copy_(bg_dev)
            flush.fill_(1)

    # ---- the autotuner's exploration of this pass (untimed), then warm-up
    def tune_step():
        restore()
        painter.fill_batch_arrays(surf, nodes, cmds, ctx=ctx)
        stream.synchronize()

    tuning = settle_tuning(ctx, tune_step)
    for _ in range(max(args.warmup, 1)):
        restore()
        painter.fill_batch_arrays(surf, nodes, cmds, ctx=ctx)
    stream.synchronize()

    # ---- timed batched steps (device-resident)
    ctx.set_timing(True)
    launches0 = ctx.launch_count
    clocks = ClockSampler(local)
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        restore()
        if world > 1:
            dist.barrier()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        painter.fill_batch_arrays(surf, nodes, cmds, ctx=ctx)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    launches = ctx.launch_count - launches0
    out_batched = surf_t.cpu().numpy()  # the last timed step's surface, for the parity check
    raster_ms, raster_n = ctx.kernel_ms("raster")
    stage = {k: ctx.kernel_ms(k)[0] / args.steps for k in ("flatten", "bins", "raster")}
    ctx.set_timing(False)
    total_ms = max_over_ranks(sum(step_ms), world, dev)
    value = replicas_value(world, mpix_step, args.steps, total_ms)

    # ---- e2e: pinned host surface through the C ABI (H2D + D2H inside)
    host_t = torch.empty(bg.size, dtype=torch.uint8, pin_memory=True)
    host = host_t.numpy()
    hsurf = Surface("rgba", W, H, host)
    e2e_s = []
    for _ in range(args.steps):
        host[:] = bg
        restore()
        if world > 1:
            dist.barrier()
        stream.synchronize()
        t0 = time.perf_counter()
        painter.fill_batch_arrays(hsurf, nodes, cmds, ctx=ctx)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = replicas_value(world, mpix_step, args.steps, max_over_ranks(1e3 * sum(e2e_s), world, dev))
    out_e2e = host.copy()
    h2d = bg.nbytes + nodes.nbytes + len(fills) * 64
    d2h = bg.nbytes

    # ---- plain per-call arm: z2dgpu_fill once per path, on the first
    # PLAIN_FILLS fills (same device-resident surface, same accounting)
    restore()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    call_us = []
    for pat, n, opts in fills[:PLAIN_FILLS]:
        t0 = time.perf_counter()
        painter.fill(surf, pat, n, opts, ctx=ctx)
        call_us.append((time.perf_counter() - t0) * 1e6)
    e1.record(stream)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_mpix = sum(px[:PLAIN_FILLS]) / 1e6
    call_us.sort()
    out_plain = surf_t.cpu().numpy()

    if rank != 0:
        clocks.stop()
        return
    peaks, peak_kind = load_peaks()
    counters = load_counters()
    build_id = source_hash()
    union_px = union_box_pixels(fills)
    alg_bytes = 2 * 4 * union_px  # read + write of every surface pixel a fill box touches
    raster_ms_per = raster_ms / max(raster_n, 1)
    achieved = alg_bytes / (raster_ms_per / 1e3) / 1e9
    arms = set(args.arms.split(",")) if args.arms not in ("all", "") else {"compositor", "breadth", "star", "jobs",
                                                                            "serving", "cpu", "png", "parity"}
    comp = comp_roof = star = jobs = None
    if "compositor" in arms:
        comp = compositor_sweep(ctx, stream, dev)
        comp_roof = {"bound": "hbm", "kernel": "k_mask_op<RGBA, src_over>", "achieved": comp["gbs_src_over"],
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": comp["gbs_src_over"] / peaks["hbm_gbs"],
                     "traffic": kernel_counter(counters, "k_mask_op_rgba_src_over_8192", "dram_bytes"),
                     "traffic_source": os.path.relpath(COUNTERS_FILE, ROOT),
                     "alg_bytes_per_launch": comp["bytes_per_px"] * 8192 * 8192, "peak_source": peak_kind}
    clk = clocks.stop()  # sampled over the batched, e2e, plain and compositor timed regions
    if comp is not None and "breadth" in arms:
        comp["breadth"] = compositor_breadth(ctx, stream, dev)
    if "star" in arms:
        star = star_latency(ctx, dev)
    if "jobs" in arms:
        jobs = jobs_arm(ctx, stream, dev)
    png_res = png_arm(ctx, surf, peaks["hbm_gbs"]) if "png" in arms else None
    serving = serving_arm(dev) if "serving" in arms else None
    # the oracle draws the whole workload (the CPU baseline) and the same
    # surfaces are compared with the GPU arms' outputs (outside any timing)
    parity = None
    if "cpu" in arms or "parity" in arms:
        cpu_v, cpu_dt, ref_all, ref_plain = cpu_sample(bg, fills, px, CPU_SAMPLE_FILLS, snapshot_at=PLAIN_FILLS)
        if CPU_SAMPLE_FILLS == N_FILLS:
            parity = {"reference": f"oracle (C++ restatement of z2d), all {N_FILLS} fills on the 4096x4096 surface",
                      "batched": diff_stats(out_batched, ref_all), "e2e": diff_stats(out_e2e, ref_all),
                      "plain": dict(diff_stats(out_plain, ref_plain), fills=PLAIN_FILLS)}
            parity["bit_exact"] = all(parity[k]["differing_bytes"] == 0 for k in ("batched", "e2e", "plain"))
    else:
        cpu_v, cpu_dt = None, 0.0
    line = {
        "metric": f"Mpix/s fill+composite (src_over, {W}x{H} RGBA, {N_FILLS} random paths)",
        "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded)",
        "config": {"workload": f"plain_large_{W}x{H}_{N_FILLS}_paths", "surface": f"rgba {W}x{H}",
                   "paths": N_FILLS, "mpix_per_step": mpix_step, "l2": "flushed (256 MiB write) before each step",
                   "mode": "batched (z2dgpu_fill_batch, device-resident surface)"},
        "summary": {
            "batched_mpix_s": value, "e2e_mpix_s": e2e_value, "plain_mpix_s": plain_mpix / (plain_ms / 1e3),
            "plain_p50_us": call_us[len(call_us) // 2],
            "star_300_p50_us": star["device"]["p50_us"] if star else None,
            "batched_over_plain": (mpix_step / (total_ms / args.steps / 1e3)) / (plain_mpix / (plain_ms / 1e3)),
            "jobs_batched_over_per_surface": (jobs["value"] / jobs["per_surface"]["value"]
                                              if jobs and jobs.get("per_surface") else None),
            "c2_bit_exact": parity["bit_exact"] if parity else None,
            "c4_bit_exact": (jobs["parity"]["differing_pixels"] == 0 if jobs and jobs.get("parity") else None),
            "c5_bit_exact": (serving["parity"]["differing_requests"] == 0
                             if serving and serving.get("parity") else None),
        },
        "stage_ms_per_step": stage,
        "plain": {"value": plain_mpix / (plain_ms / 1e3), "unit": "Mpix/s", "ms": plain_ms,
                  "calls": PLAIN_FILLS, "note": f"z2dgpu_fill per path, first {PLAIN_FILLS} fills",
                  "latency_us": {"p50": call_us[len(call_us) // 2], "p99": call_us[int(len(call_us) * 0.99) - 1],
                                 "note": "host wall time per painter.fill call, Python marshalling included (a "
                                         "short path returns once its one upload and raster launch are queued; "
                                         "a longer one after the pipeline's size readbacks)"}},
        "star_300": star,
        "jobs": jobs,
        "serving": serving,
        "png": png_res,
        "autotune": tuning,
        "batched_over_plain": (mpix_step / (total_ms / args.steps / 1e3)) / (plain_mpix / (plain_ms / 1e3)),
        "parity": parity,
        "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": "k_raster", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "traffic": kernel_counter(counters, "k_raster", "dram_bytes"),
                     "traffic_source": os.path.relpath(COUNTERS_FILE, ROOT),
                     "traffic_build": counters.get("source_hash") if counters else None, "build": build_id,
                     "peak_source": peak_kind, "alg_bytes_per_launch": alg_bytes,
                     "launch_ms": raster_ms_per},
        "compute_roofline": issue_roofline(counters, raster_ms_per, clk),
        "cpu_baseline": {"value": cpu_v, "unit": "Mpix/s", "cores": 1, "kind": "port",
                         "sample": f"first {CPU_SAMPLE_FILLS} of {N_FILLS} fills, {cpu_dt:.1f} s"},
        "compositor": comp,
        "compositor_roofline": comp_roof,
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--arms", default="all",
                    help="extra arms beside the batched / e2e / per-call fill arms: 'all', 'none' or a comma "
                         "list of compositor, breadth, star, jobs, serving, cpu, png, parity (shorter runs for profiling)")
    ap.add_argument("--jobs", type=int, default=4096,
                    help="surfaces of the batched-jobs arm (smaller for profiling captures)")
    ap.add_argument("--size", type=int, default=4096,
                    help="side of the fill workload's surface (smaller only for profiling captures)")
    ap.add_argument("--fills", type=int, default=2000,
                    help="paths of the fill workload (smaller only for profiling captures)")
    ap.add_argument("--breadth-size", type=int, default=8192,
                    help="side of the compositor breadth arm's surfaces (smaller only for profiling captures)")
    ap.add_argument("--breadth-only", default="",
                    help="run only the breadth cells whose name contains this, e.g. linear/linear_rgb/none")
    ap.add_argument("--counters-from", action="append", default=[], metavar="NAME=CSV",
                    help="write the per-launch counters file from ncu --csv captures and exit")
    args = ap.parse_args()
    if args.counters_from:
        write_counters(args.counters_from)
        return
    globals()["N_JOBS"] = args.jobs
    globals()["BREADTH_SIZE"] = args.breadth_size
    globals()["BREADTH_ONLY"] = args.breadth_only
    globals()["W"] = globals()["H"] = args.size
    globals()["N_FILLS"] = globals()["CPU_SAMPLE_FILLS"] = args.fills
    globals()["PLAIN_FILLS"] = min(PLAIN_FILLS, args.fills)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
