"""The multi-rank path of bench.py on CPU: two gloo ranks, max-over-ranks timing.

The engine runs one replica per GPU (the reference has no multi-GPU code and
the workload needs no exchange), so the only cross-rank logic is the barrier
and the maximum of the per-rank step times.
"""

from __future__ import annotations

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    dist.barrier()
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank])
    out[rank] = got
    dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    world = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    assert out[0] == [2.0, 10.0]
    assert out[1] == [2.0, 10.0]


def test_single_process_passthrough_and_replica_value():
    import bench

    assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    assert bench.replica_value(1000.0, 2.0, 4) == pytest.approx(4 * 1000.0 / 2e-3)
