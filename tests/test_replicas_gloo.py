"""Replica aggregation across 2 ranks with the gloo backend on CPU: the job
time is the slowest rank's, throughput counts every rank's work."""
import os

import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bdda.replicas import job_throughput, max_over_ranks
    t = max_over_ranks(1.0 + rank)
    out[rank] = (t, job_throughput(16.0, t, world))
    dist.destroy_process_group()


def test_two_rank_gloo_aggregation():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == (2.0, 16.0)


def test_single_process_fallback():
    from bdda.replicas import job_throughput, max_over_ranks
    assert max_over_ranks(3.5) == 3.5
    assert job_throughput(10.0, 2.0, 1) == pytest.approx(5.0)
