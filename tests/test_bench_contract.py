"""bench.py's output contract on the CPU: the reference arm's JSON line (the
driver reads it at every round end) and the per-launch counters file that
the GPU arm's roofline reads (written from ncu CSV captures, tagged with the
source hash of the kernels it describes)."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"] == "plain_large_4096x4096_2000_paths"


def _ncu_csv(path, kernel, metrics):
    head = ('"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size","Grid Size",'
            '"Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"')
    rows = [head]
    for launch in (0, 1):
        for name, value in metrics.items():
            rows.append(f'"{launch}","1","python3","host","{kernel}","1","7","(128, 1, 1)","(16368, 1, 1)","0",'
                        f'"10.3","Command line profiler metrics","{name}","byte","{value + launch}"')
    with open(path, "w") as f:
        f.write("==PROF== preamble\n" + "\n".join(rows) + "\n")


def test_counters_file_merges_captures(tmp_path, monkeypatch):
    import bench
    monkeypatch.setattr(bench, "COUNTERS_FILE", str(tmp_path / "counters.json"))
    a, b = tmp_path / "d.csv", tmp_path / "i.csv"
    _ncu_csv(a, "void k_raster<0, 1>(RasterArgs)", {"dram__bytes_read.sum": 1000, "dram__bytes_write.sum": 200,
                                                     "gpu__time_duration.sum": 4000})
    _ncu_csv(b, "void k_raster<0, 1>(RasterArgs)", {"smsp__inst_executed.sum": 5000, "gpu__time_duration.sum": 4100})
    bench.write_counters([f"k_raster={a}", f"k_raster={b}"])
    out = bench.load_counters()
    assert out["source_hash"] == bench.source_hash()
    k = out["kernels"]["k_raster"]
    # the last launch of each capture; captures of one kernel merge
    assert k["dram_read"] == 1001 and k["dram_write"] == 201 and k["dram_bytes"] == 1202
    assert k["inst_executed"] == 5001 and k["duration_ns"] == 4101
    assert k["captures"] == ["d.csv", "i.csv"]
    assert bench.kernel_counter(out, "k_raster", "inst_executed") == 5001
    assert bench.kernel_counter(out, "k_mask_op", "dram_bytes") is None


def test_counters_file_of_another_source_is_replaced(tmp_path, monkeypatch):
    import bench
    path = tmp_path / "counters.json"
    monkeypatch.setattr(bench, "COUNTERS_FILE", str(path))
    path.write_text(json.dumps({"source_hash": "0" * 16, "kernels": {"old": {"dram_bytes": 1}}}))
    a = tmp_path / "d.csv"
    _ncu_csv(a, "k_mask_op<3, 3>", {"dram__bytes_read.sum": 10, "dram__bytes_write.sum": 5})
    bench.write_counters([f"k_mask_op_rgba_src_over_8192={a}"])
    out = bench.load_counters()
    assert set(out["kernels"]) == {"k_mask_op_rgba_src_over_8192"}
    assert out["kernels"]["k_mask_op_rgba_src_over_8192"]["dram_bytes"] == 17
