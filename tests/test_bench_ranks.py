"""bench.py's multi-rank path on the CPU (gloo, world size 2): every rank
runs a replica of the workload, the job's time is the slowest rank's
(max_over_ranks, one all-reduce), the value is the whole job's
(replicas_value), and the reference arm prints from rank 0 only."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
        total = bench.max_over_ranks(ms, world, "cpu")
        q.put((rank, total, bench.replicas_value(world, 10.0, 4, total)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; 2 replicas x 10 Mpix x 4 steps in 0.15 s
    assert [t for _, t, _ in got] == [150.0, 150.0]
    assert all(abs(v - 2 * 10.0 * 4 / 0.15) < 1e-9 for _, _, v in got)


def test_single_rank_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.replicas_value(1, 629.0, 5, 5000.0) == pytest.approx(629.0)


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
