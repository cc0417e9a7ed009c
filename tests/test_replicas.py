"""Multi-GPU runs are replicas (every rank solves its own copy of the batch; no collective on the data path):
the host logic of bench.py across ranks, on the CPU with the gloo backend (world size 2)."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, v = bench.replicas_rate(1.0 + rank, 256, world, dist, "cpu")
    q.put((rank, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_the_slowest_replica_sets_the_job_rate():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in out:
        assert t == 2.0 and v == pytest.approx(world * 256 / 2.0)


def test_single_rank_rate_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replicas_rate(4.0, 256, 1) == (4.0, 64.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(None)            # returns before touching its arguments
    assert capsys.readouterr().out == ""
