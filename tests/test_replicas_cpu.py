"""CPU: the multi-rank path of bench.py (one independent replica per rank,
no data-path collective) -- the barrier-bracketed timing takes the slowest
rank's time and the job's throughput sums the replicas.  world_size 2 over
gloo on 127.0.0.1."""

import os
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        # rank r "took" 1 + r seconds for its steps
        t = bench.max_over_ranks(dist, 1.0 + rank, "cpu")
        out[rank] = t
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    world = 2
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        assert dict(out) == {0: 2.0, 1: 2.0}


def test_replica_throughput_sums_replicas():
    sys.path.insert(0, ROOT)
    import bench

    # 684.7 GF per step, 2 replicas, slowest 0.25 s -> 5.4776 TFLOP/s
    assert bench.replica_throughput(684.7e9, 2, 0.25) == pytest.approx(5.4776)
    assert bench.replica_throughput(684.7e9, 1, 0.25) == pytest.approx(2.7388)
