"""The z-slab decomposition (stzpp_gb300/slabs.py) with GPU sub-domains.

Several slabs on one GPU, each a handle over its planes and ghost planes,
exchanging planes through device buffers (LocalTransport), against one
handle over the whole grid: the fine level's x bit for bit after two
decomposed sweeps and after a two-level cycle (restriction gathered onto the
root, coarse correction broadcast and interpolated), the residual norm to
1e-13.  Dirichlet and periodic z, 2-4 slabs.  Runs on one GPU: the slabs
exchange through copies, not through kernels waiting on one another.
"""
import numpy as np
import pytest

from oracle import problem as P

pytestmark = pytest.mark.gpu

CASES = [((64, 64, 41), False, 2), ((64, 32, 40), False, 3), ((32, 32, 32), True, 2), ((64, 64, 48), True, 4)]


def coarse_solve(rc):
    return 1e-3 * rc + 1e-4


@pytest.mark.parametrize("dims,zp,parts", CASES)
def test_gpu_slabs_are_the_undivided_level(dims, zp, parts):
    import torch
    import stzpp_gb300 as sg
    from stzpp_gb300 import slabs as SL
    m, n, o = dims
    per = (True, True, zp)
    h = P.grid_spacing(m, n, o, per)
    st, fix = sg.elastic_stencil(1.0, 2.0, *h)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((o, n, m, 3))
    r = rng.standard_normal((o, n, m, 3))
    # the undivided level: a handle over the whole grid, two levels
    with sg.Multigrid(dims, per, precision="fp64", bottom="gs", max_coarse=m * n * o - 1) as ref:
        ref.setup_matrices(stencil=st, fix=fix)
        ref.level_set_field(0, "x", x.reshape(-1, 3))
        ref.level_set_field(0, "r", r.reshape(-1, 3))
        ref.gauss_seidel(0, 2)
        x_sweep = ref.level_get_field(0, "x").reshape(o, n, m, 3)
        _, sq = ref.residual(0)
        ref.restriction(1)
        rc = ref.level_get_field(1, "r")
        ref.level_set_field(1, "x", coarse_solve(rc))
        ref.interpolation(1)
        ref.gauss_seidel(0, 2)
        x_cycle = ref.level_get_field(0, "x").reshape(o, n, m, 3)

    def make(L):
        s = SL.HandleSlab((m, n), (True, True), L, st, fix)
        ks = [(L.first + i) % o for i in range(L.nplanes)]
        s.set_planes(0, "x", 0, torch.from_numpy(np.ascontiguousarray(x[ks].reshape(-1, 3))).cuda())
        s.set_planes(0, "r", 0, torch.from_numpy(np.ascontiguousarray(r[ks].reshape(-1, 3))).cuda())
        return s

    def owned(solver):
        out = {}
        for p, L in enumerate(solver.layouts):
            out[p] = solver.slabs[p].get_planes(0, "x", L.local(L.k0), L.k1 - L.k0).cpu().numpy()
        return out

    for cycle in (False, True):
        solver = SL.SlabSolver.split(o, zp, parts, make, SL.LocalTransport(parts))
        try:
            if cycle:
                solver.two_level_cycle(2, 2, lambda rc_: coarse_solve(rc_))
                want = x_cycle
            else:
                solver.sweep(2)
                want = x_sweep
                got_sq = solver.residual()
                assert abs(got_sq - sq) <= 1e-13 * sq
            got = owned(solver)
            for p, L in enumerate(solver.layouts):
                assert np.array_equal(got[p], want[L.k0:L.k1].reshape(-1, 3)), (cycle, p)
        finally:
            for s in solver.slabs.values():
                s.close()
