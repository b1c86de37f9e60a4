"""Host logic of the multi-GPU bench: every rank is an independent replica
(the path has no cross-lattice exchange); the slowest rank's time is the job's
time.  Two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        q.put((rank, bench.ranks_max(1.5 + rank, dist)))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert got == [(0, 2.5), (1, 2.5)]


def test_replica_device_selection():
    assert bench.replica_device({"WORLD_SIZE": "4", "LOCAL_RANK": "3"}) == "3"
    assert bench.replica_device({"WORLD_SIZE": "4", "LOCAL_RANK": "3", "CUDA_VISIBLE_DEVICES": "5"}) is None
    assert bench.replica_device({}) is None
    assert bench.ranks_max(3.0, None) == 3.0
