"""The N > 1 path on the CPU: replicas with no data exchange, meeting only in the timing reduction.

Two gloo ranks check reduce_timing (slowest rank's time, summed units) and that every rank computes the
same disjoint scene split; the reference arm under torchrun with two ranks prints exactly one line (rank 0)
and every rank exits 0.
"""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

from mpm_plugin_gb300.replicas import aggregate_rate, reduce_timing, shard

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_is_a_balanced_partition():
    costs = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0, 1.0, 4.0]
    for world in (1, 2, 3, 4):
        parts = [shard(costs, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs)
    assert shard([], 0, 2) == []


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    t, u = reduce_timing(1.0 + rank, 100.0 * (rank + 1))
    rate = aggregate_rate(2.0 - rank, 10.0)
    split = shard([3.0, 1.0, 4.0, 1.0, 5.0, 9.0, 2.0], rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, split)
    dist.barrier()
    Path(out_dir, f"{rank}.json").write_text(json.dumps({"t": t, "u": u, "rate": rate, "splits": gathered}))
    dist.destroy_process_group()


def test_reduce_timing_over_two_gloo_ranks(tmp_path):
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, start_method="spawn")
    res = [json.loads((tmp_path / f"{r}.json").read_text()) for r in range(2)]
    for r in res:
        assert r["t"] == 2.0 and r["u"] == 300.0  # slowest rank; units of both
        assert r["rate"] == pytest.approx(20.0 / 2.0)
        a, b = r["splits"]
        assert not set(a) & set(b) and sorted(a + b) == list(range(7))
    assert res[0]["splits"] == res[1]["splits"]


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
