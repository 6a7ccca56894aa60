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


def test_clock_samples_are_taken_from_the_timed_region():
    """bench.py's clock record keeps the nvidia-smi samples stamped inside the
    timed region, reports the throttle reasons seen there, and falls back to
    every sample when no stamp falls in the window."""
    import datetime

    import bench
    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5, 100000)
    t1 = t0 + datetime.timedelta(milliseconds=300)

    def line(ms, sm, thermal="Not Active", cap="Not Active"):
        ts = (t0 + datetime.timedelta(milliseconds=ms)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return f"{ts}, 0, {sm}, 2070, 900.5, 0x0, Not Active, Not Active, {thermal}, {cap}\n"

    lines = [line(-500, 1200, thermal="Active"),   # warm-up: a slowdown outside the window
             line(50, 2070), line(120, 2055, cap="Active"), line(250, 2070),
             line(900, 1500)]                       # after the timed region
    got = bench.Clocks.summarise(lines, t0, t1)
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3,
                   "window": "timed region"}
    late = bench.Clocks.summarise(lines, t1 + datetime.timedelta(seconds=10), t1 + datetime.timedelta(seconds=11))
    assert late["samples"] == 5 and late["window"].startswith("sampler lifetime")
    assert "sw_thermal_slowdown" in late["reasons"]
    assert bench.Clocks.summarise(["garbage\n"], t0, t1) is None
