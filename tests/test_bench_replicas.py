"""bench.py's multi-rank path on CPU (gloo, world size 2).

On a GPU node `bench.py --gpus N` runs under torchrun as N independent
replicas: no collective on the data path, only a barrier around the timed
region and a max (time) / sum (steps) over ranks for the reported value.
These tests run that host logic with two gloo ranks, and the reference arm
under torchrun, where rank 0 alone works and prints one JSON line."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _ranks(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local, pg = bench.dist_init(world)
    assert (r, w, local) == (rank, world, rank) and pg is not None
    bench.barrier(pg)
    t_max = bench.max_over_ranks(pg, 1.0 + rank)      # the slowest rank's time
    n_sum = bench.sum_over_ranks(pg, 10.0 * (rank + 1))  # every rank's steps
    out.put((rank, t_max, n_sum))
    pg.destroy_process_group()


def test_replica_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ranks, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "16", "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2
    assert d["config"]["parallelism"] == "replicas x2"
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
