"""The z-slab decomposition (stzpp_gb300/slabs.py) on the CPU.

Sub-domains are numpy levels (oracle/slab_numpy.py), so these tests check
the decomposition itself -- the partition, the two ghost-plane exchanges per
sweep, the residual norm's all-reduce, the restriction gathered onto the
root and the interpolation of the broadcast correction -- against the same
numpy operations on the undivided grid: x bit for bit after sweeps and
after a two-level cycle, the norm to 1e-13.  In one process
(LocalTransport, 2-4 slabs) and on two gloo ranks (DistTransport).
"""
import os
import socket

import numpy as np
import pytest

from oracle import problem as P
from oracle.slab_numpy import NumpyLevel
from stzpp_gb300 import slabs as SL

CASES = [((8, 8, 24), True, 2), ((8, 8, 24), True, 3), ((8, 6, 25), False, 2), ((8, 6, 33), False, 4),
         ((6, 8, 20), False, 3)]


def setup_case(dims, zp, seed=5):
    m, n, o = dims
    h = (1.0 / m, 1.0 / n, 1.0 / (o if zp else o - 1))
    st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((o, n, m, 3))
    r = rng.standard_normal((o, n, m, 3))
    return st, fix, x, r


def make_slab(dims, zp, st, fix, x, r, L):
    m, n, o = dims
    s = NumpyLevel(m, n, L.nplanes, False, st, fix)
    ks = [(L.first + i) % o for i in range(L.nplanes)]
    s.f["x"][:] = x[ks]
    s.f["r"][:] = r[ks]
    return s


def owned_x(solver):
    out = {}
    for p in solver.t.mine():
        L = solver.layouts[p]
        out[p] = solver.slabs[p].f["x"][L.local(L.k0):L.local(L.k0) + L.k1 - L.k0]
    return out


def coarse_solve(rc):
    """Any fixed map of the coarse right-hand side serves to follow the data."""
    return 1e-3 * rc + 1e-4


def reference_cycle(dims, zp, st, fix, x, r, sweeps):
    m, n, o = dims
    ref = NumpyLevel(m, n, o, zp, st, fix)
    ref.f["x"][:] = x
    ref.f["r"][:] = r
    for _ in range(sweeps):
        ref.colours(0, 8)
    x_sweep = ref.f["x"].copy()
    ref.residual()
    sq = float((ref.f["res"] ** 2).sum())
    ref.restrict()
    ref.cf["x"] = coarse_solve(ref.cf["r"].reshape(-1, 3)).reshape(ref.cf["r"].shape)
    ref.interpolate()
    for _ in range(sweeps):
        ref.colours(0, 8)
    return x_sweep, sq, ref.f["x"].copy()


def test_partition_and_layout():
    assert SL.partition(257, False, 4) == [(0, 64), (64, 128), (128, 192), (192, 257)]
    assert SL.partition(24, True, 3) == [(0, 8), (8, 16), (16, 24)]
    for o, zp, P_ in ((257, False, 4), (24, True, 3), (25, False, 2), (20, False, 3)):
        for k0, k1 in SL.partition(o, zp, P_):
            L = SL.SlabLayout(o, zp, k0, k1)
            assert L.first % 2 == 0 and L.local(k0) >= (1 if L.lo else 0)
            assert L.local(k1 - 1) + (1 if L.hi else 0) == L.nplanes - 1
            if L.lo:
                assert L.local((k0 - 1) % o) == L.local(k0) - 1
    with pytest.raises(ValueError):
        SL.partition(10, False, 3)
    with pytest.raises(ValueError):
        SL.partition(25, True, 2)


@pytest.mark.parametrize("dims,zp,parts", CASES)
def test_decomposed_sweeps_and_cycle_are_the_undivided_ones(dims, zp, parts):
    st, fix, x, r = setup_case(dims, zp)
    o = dims[2]
    solver = SL.SlabSolver.split(o, zp, parts, lambda L: make_slab(dims, zp, st, fix, x, r, L),
                                 SL.LocalTransport(parts))
    x_sweep, sq, x_cycle = reference_cycle(dims, zp, st, fix, x, r, 2)
    solver.sweep(2)
    got = owned_x(solver)
    for p, L in enumerate(solver.layouts):
        assert np.array_equal(got[p], x_sweep[L.k0:L.k1]), p
    assert abs(solver.residual() - sq) <= 1e-13 * sq
    # the two-level cycle from the same start
    solver = SL.SlabSolver.split(o, zp, parts, lambda L: make_slab(dims, zp, st, fix, x, r, L),
                                 SL.LocalTransport(parts))
    solver.two_level_cycle(2, 2, coarse_solve)
    got = owned_x(solver)
    for p, L in enumerate(solver.layouts):
        assert np.array_equal(got[p], x_cycle[L.k0:L.k1]), p


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, dims, zp, results):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        st, fix, x, r = setup_case(dims, zp)
        t = SL.DistTransport()
        solver = SL.SlabSolver.split(dims[2], zp, world, lambda L: make_slab(dims, zp, st, fix, x, r, L), t)
        solver.sweep(2)
        sq = solver.residual()
        results[("sweep", rank)] = owned_x(solver)[rank].copy()
        results[("sq", rank)] = sq
        solver = SL.SlabSolver.split(dims[2], zp, world, lambda L: make_slab(dims, zp, st, fix, x, r, L), t)
        solver.two_level_cycle(2, 2, coarse_solve)
        results[("cycle", rank)] = owned_x(solver)[rank].copy()
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("dims,zp", [((8, 8, 24), True), ((8, 6, 25), False)])
def test_two_gloo_ranks(dims, zp):
    """Two processes, one slab each, exchanging through gloo: the same x as
    the undivided grid, bit for bit, and the same all-reduced norm on both."""
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as manager:
        results = manager.dict()
        mp.spawn(_worker, args=(2, port, dims, zp, results), nprocs=2, join=True)
        got = dict(results)
    st, fix, x, r = setup_case(dims, zp)
    x_sweep, sq, x_cycle = reference_cycle(dims, zp, st, fix, x, r, 2)
    for p, (k0, k1) in enumerate(SL.partition(dims[2], zp, 2)):
        assert np.array_equal(got[("sweep", p)], x_sweep[k0:k1])
        assert np.array_equal(got[("cycle", p)], x_cycle[k0:k1])
    assert got[("sq", 0)] == got[("sq", 1)]
    assert abs(got[("sq", 0)] - sq) <= 1e-13 * sq
