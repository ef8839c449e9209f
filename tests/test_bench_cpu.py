"""The benchmark's host logic on CPU: the whole-job rate over ranks (gloo,
two processes) and the reference arm under torchrun, where rank 0 alone
times the CPU implementation and prints the line."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 * (rank + 1)
    out[rank] = (bench.max_over_ranks(ms), bench.whole_job_rate(1000, 5, ms, world))
    dist.destroy_process_group()


def test_whole_job_rate_over_gloo_ranks():
    import torch.multiprocessing as mp
    port = free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    # the slowest rank (20 ms) sets the time; every rank's particles count
    for r in (0, 1):
        assert res[r][0] == 20.0
        assert abs(res[r][1] - 2 * 1000 * 5 / 0.020) < 1e-6


def test_single_process_rate():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10, 4, 2.0, 1) == 10 * 4 / 0.002


def test_error_and_latency_summaries():
    import numpy as np
    import bench
    ref = np.zeros((4, 3))
    got = np.array([[0, 0, 0], [3e-4, 0, 0], [0, 4e-4, 0], [0, 0, 1.0]])
    e = bench.position_error(got, ref, radius=0.5)
    assert e["max"] == 1.0 and e["frac_above_1e-3_radius"] == 0.25
    assert abs(e["median"] - 3.5e-4) < 1e-12
    p = bench.percentiles([1.0, 2.0, 3.0, 4.0])
    assert p["p50"] == 2.5 and p["p99"] <= 4.0


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun():
    env = dict(os.environ, BCS_REFERENCE_BUDGET_S="1", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--cells-per-type", "60"]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=580, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                      # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
