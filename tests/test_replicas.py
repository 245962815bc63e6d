"""The multi-GPU form of bench.py is independent replicas: N ranks each run the
whole domain, with a barrier around the timed region and the maximum time over
the ranks, and no collective on the data path.  These tests run that host
logic on CPU ranks over gloo (world size 2)."""
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


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    ws, r, _ = bench.dist_init()
    bench.barrier(ws)
    t = bench.max_over_ranks(ws, 1.0 + r)     # each rank's own "timed region"
    q.put((r, ws, t))
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_on_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(o[0] for o in out) == [0, 1]
    assert all(o[1] == 2 and o[2] == 2.0 for o in out)


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    """bench.py --impl reference under torchrun with 2 ranks: rank 0 times the
    CPU oracle on a small grid and prints one JSON line; rank 1 exits 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "16", "8", "8", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, env=env, timeout=280)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["steps"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0
