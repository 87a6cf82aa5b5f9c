"""The N>1 path of bench.py (replicas only: no data-path collective) on CPU with gloo, world
size 2: the timing is the slowest rank's, and the job value counts every rank's iterations."""
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
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        out[rank] = t
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_bench_replicas_max_over_ranks_gloo():
    import bench
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: 2.5, 1: 2.5}
    # two replicas of 3 steps each in 6 s: 1 s per iteration of the whole job
    assert bench.job_seconds_per_iter(6.0, 3, 2) == pytest.approx(1.0)
    assert bench.max_over_ranks(0.25, None) == 0.25
