"""The bench's multi-rank logic on CPU ranks (gloo, world size 2): every
rank gets the slowest rank's time, the whole-job rate counts every rank's
units over that time, and under torchrun the reference arm prints one line
from rank 0 while the other rank exits without work."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        ms = bench.max_over_ranks(times[rank], world, "cpu")
        out.put((rank, ms, bench.whole_job_rate(10, world, ms)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [10.0, 25.0]
    mp.start_processes(_rank, args=(2, free_port(), times, q), nprocs=2, join=True, start_method="spawn")
    got = sorted(q.get(timeout=30) for _ in range(2))
    assert [g[1] for g in got] == [25.0, 25.0]                # the slowest rank's time on both
    assert all(abs(g[2] - 10 * 2 / 0.025) < 1e-6 for g in got)  # 800 units/s over both ranks
    import bench
    assert bench.max_over_ranks(7.0, 1, "cpu") == 7.0


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, env=env, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, res.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_unknown_workload_names_are_an_argument_error():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--configs",
                        "roundtrip,cfg1"], capture_output=True, text=True, cwd=ROOT)
    assert p.returncode == 2
    assert "unknown workload(s) cfg1" in p.stderr
