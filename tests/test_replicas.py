"""The multi-GPU form of the bench is replicas only (one independent system
per rank, no collective on the data path): the job's figure is the sum of
the replicas' particle-steps at the pace of the slowest.  The aggregation
runs here on two CPU processes over gloo."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [12.5, 20.0][rank]  # rank 1 is the slow replica
    ms_max = bench.replica_max(ms, dist, "cpu")
    out[rank] = (ms_max, bench.job_value(1000, world, ms_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_pace():
    world = 2
    with mp.get_context("spawn").Manager() as mgr:  # no fork of this (threaded) process
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ms_max, value = res[rank]
        assert ms_max == 20.0
        assert value == pytest.approx(2 * 1000 / 0.020)


def test_single_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_max(7.0, None, "cpu") == 7.0
    assert bench.job_value(4194304, 1, 18.0) == pytest.approx(4194304 / 0.018)
