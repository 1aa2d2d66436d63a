"""Multi-GPU form = replicas only: the bench's per-rank stream seeds are disjoint and
the job time is the slowest rank's, checked with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out[rank] = (bench.max_over_ranks(1.5 + rank, world), bench.replica_seeds(rank, 4))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_disjoint_seeds():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 2.5
    assert not set(out[0][1]) & set(out[1][1])
    import bench
    assert bench.max_over_ranks(3.0, 1) == 3.0
