"""Replica aggregation of bench.py over two gloo ranks on the CPU (127.0.0.1)."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, units = bench.reduce_over_ranks(1.0 + rank, 100 * (rank + 1), torch.device("cpu"))
    out[rank] = (t, units)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn",
                       join=True)
    # every rank sees the slowest rank's time and the units of all ranks
    assert dict(out) == {0: (2.0, 300), 1: (2.0, 300)}
