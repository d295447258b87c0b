"""The multi-rank host path of bench.py with two gloo ranks on CPU: each rank
is an independent replica; the job time is the slowest rank's and the units
are summed (no collective on the data path)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units, value = bench.aggregate_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1))
    out[rank] = (ms, units, value, bench.dist_env())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_replicas():
    world, port = 2, _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    for rank in range(world):
        ms, units, value, env = out[rank]
        assert ms == 15.0 and units == 3000.0
        assert value == pytest.approx(3000.0 / 0.015)
        assert env == (world, rank, 0)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_ranks(4.0, 100) == (4.0, 100.0, 100 / 0.004)
