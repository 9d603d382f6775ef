"""bench.py's multi-GPU path is replicas only: each rank solves its own copy and the
job time is the max over ranks, the work the sum.  Checked with world_size 2 on gloo."""
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


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units = bench.aggregate_replicas(100.0 + 50.0 * rank, 1000 * (rank + 1), dist, "cpu")
    out[rank] = (ms, units)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for r in range(2):
        assert out[r] == (150.0, 3000.0)


def test_single_rank_passthrough():
    import bench
    assert bench.aggregate_replicas(12.5, 77) == (12.5, 77.0)
