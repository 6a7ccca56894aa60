"""The N>1 path of bench.py: independent replicas, one per rank, timed as the
max over ranks (the solve itself is not sharded).  Two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, results):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    per_rank_ms = [10.0, 14.5][rank]
    m = bench.reduce_max(per_rank_ms, dist, "cpu")
    results[rank] = (m, bench.job_ms_per_solve(m, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as manager:
        results = manager.dict()
        mp.spawn(_worker, args=(2, port, results), nprocs=2, join=True)
        got = dict(results)
    assert got[0] == got[1] == (14.5, 7.25)


def test_single_process_reduction_is_identity():
    import bench
    assert bench.reduce_max(3.0, None, "cpu") == 3.0
    assert bench.job_ms_per_solve(3.0, 1) == 3.0
