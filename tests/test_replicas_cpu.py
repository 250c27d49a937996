"""bench.py's multi-GPU path runs independent replicas: the job time is the
slowest rank's (all-reduce MAX) and the value counts every rank's updates.
Checked with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    t = bench.replica_max(local_ms, "cpu")
    out.put((rank, t, bench.replica_value(world, 1000, 10, t)))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, value in res:
        assert t == 150.0
        assert value == pytest.approx(2 * 1000 * 10 / 0.150)
