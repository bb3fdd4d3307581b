"""The N > 1 path of bench.py on CPU: two processes joined over gloo (no GPU).
Each rank stands for one replica; the job time is the slowest rank's and the
job throughput counts every rank's units (weak scaling, no collective on the
data path -- the path shards by independent transforms)."""
import os
import socket

import pytest


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def worker(rank, world, port, results):
    import torch
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 10 + r ms for its replica of the workload
        ms = bench.max_over_ranks(10.0 + rank, world, torch.device("cpu"))
        value = bench.job_throughput(2.0e9, world, ms)
        results[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo():
    import torch.multiprocessing as mp
    port = free_port()
    mgr = mp.Manager()
    results = mgr.dict()
    mp.spawn(worker, args=(2, port, results), nprocs=2, join=True)
    assert set(results.keys()) == {0, 1}
    for rank in (0, 1):
        ms, value = results[rank]
        assert ms == pytest.approx(11.0)                      # the slowest rank
        assert value == pytest.approx(2.0e9 * 2 / 11e-3 / 1e9)  # both ranks' units
