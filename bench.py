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
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch,
# from the ncu captures summarised under profiles/
TRAFFIC = {
    "k_raster": (214_508_288, "profiles/k_raster_rgba4096_2000paths.md"),
    "k_mask_op": (544_317_696, "profiles/k_mask_op_rgba8192_src_over.md"),
}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


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
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
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


def cpu_sample(bg, fills, px, n_fills):
    from oracle import Oracle
    from z2d_gb300.surface import Surface
    o = Oracle()
    s = Surface("rgba", W, H, bg.copy())
    t0 = time.perf_counter()
    for pat, nodes, opts in fills[:n_fills]:
        o.fill(s, pat, nodes, opts)
    dt = time.perf_counter() - t0
    return sum(px[:n_fills]) / 1e6 / dt, dt


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

    # ---- warm-up
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
    raster_ms, raster_n = ctx.kernel_ms("raster")
    ctx.set_timing(False)
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * mpix_step * args.steps / (total_ms / 1e3)

    # ---- e2e: pinned host surface through the C ABI (H2D + D2H inside)
    host_t = torch.empty(bg.size, dtype=torch.uint8, pin_memory=True)
    host = host_t.numpy()
    hsurf = Surface("rgba", W, H, host)
    e2e_s = []
    for _ in range(args.steps):
        host[:] = bg
        restore()
        stream.synchronize()
        t0 = time.perf_counter()
        painter.fill_batch_arrays(hsurf, nodes, cmds, ctx=ctx)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = mpix_step * args.steps / sum(e2e_s)
    h2d = bg.nbytes + nodes.nbytes + len(fills) * 64
    d2h = bg.nbytes

    # ---- plain per-call arm: z2dgpu_fill once per path, on the first
    # PLAIN_FILLS fills (same device-resident surface, same accounting)
    restore()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for pat, n, opts in fills[:PLAIN_FILLS]:
        painter.fill(surf, pat, n, opts, ctx=ctx)
    e1.record(stream)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_mpix = sum(px[:PLAIN_FILLS]) / 1e6

    if rank != 0:
        clocks.stop()
        return
    peaks, peak_kind = load_peaks()
    union_px = union_box_pixels(fills)
    alg_bytes = 2 * 4 * union_px  # read + write of every surface pixel a fill box touches
    raster_ms_per = raster_ms / max(raster_n, 1)
    achieved = alg_bytes / (raster_ms_per / 1e3) / 1e9
    comp = compositor_sweep(ctx, stream, dev)
    clk = clocks.stop()  # sampled over the batched, e2e, plain and compositor timed regions
    comp_roof = {"bound": "hbm", "kernel": "k_mask_op<RGBA, src_over>", "achieved": comp["gbs_src_over"],
                 "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": comp["gbs_src_over"] / peaks["hbm_gbs"],
                 "traffic": TRAFFIC["k_mask_op"][0], "traffic_source": TRAFFIC["k_mask_op"][1],
                 "alg_bytes_per_launch": comp["bytes_per_px"] * 8192 * 8192, "peak_source": peak_kind}
    cpu_v, cpu_dt = cpu_sample(bg, fills, px, CPU_SAMPLE_FILLS)
    line = {
        "metric": "Mpix/s fill+composite (src_over, 4096x4096 RGBA, 2000 random paths)",
        "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded)",
        "config": {"workload": "plain_large_4096x4096_2000_paths", "surface": "rgba 4096x4096",
                   "paths": N_FILLS, "mpix_per_step": mpix_step, "l2": "flushed (256 MiB write) before each step",
                   "mode": "batched (z2dgpu_fill_batch, device-resident surface)"},
        "plain": {"value": plain_mpix / (plain_ms / 1e3), "unit": "Mpix/s", "ms": plain_ms,
                  "calls": PLAIN_FILLS, "note": f"z2dgpu_fill per path, first {PLAIN_FILLS} fills"},
        "batched_over_plain": (mpix_step / (total_ms / args.steps / 1e3)) / (plain_mpix / (plain_ms / 1e3)),
        "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": "k_raster", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": TRAFFIC["k_raster"][0],
                     "traffic_source": TRAFFIC["k_raster"][1],
                     "peak_source": peak_kind, "alg_bytes_per_launch": alg_bytes,
                     "launch_ms": raster_ms_per},
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
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
