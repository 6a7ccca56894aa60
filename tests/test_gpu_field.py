"""The steps on either side of the solve, on the GPU, against the oracle's
restatements: the right-hand side assembly (node divergence of the cell tensor
field, calculate_first_order_stresses) and the projection-step stress update
(calculate_first_order_velocities and the stress increments) -- bit-identical
(same operation order, no FMA contraction)."""
import numpy as np
import pytest

from oracle import problem as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,per", [((16, 16, 17), (True, True, False)), ((12, 10, 9), (False, False, False)),
                                      ((8, 6, 10), (True, False, True)), ((32, 32, 33), (True, True, False))])
def test_rhs_divergence_bit_exact(dims, per):
    import stzpp_gb300 as sg
    from stzpp_gb300 import problems
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    eps = problems.random_strain(3, dims, per)
    ref = P.rhs_divergence(eps, m, n, o, per, *h)
    with sg.Multigrid(dims, per, max_coarse=10**9) as mg:
        mg.set_rhs_divergence(eps, h)
        got = mg.get_rhs()
    assert np.array_equal(got, ref), np.abs(got - ref).max()


@pytest.mark.parametrize("dims,per", [((16, 16, 17), (True, True, False)), ((12, 10, 9), (False, False, False)),
                                      ((16, 12, 8), (True, False, True))])
@pytest.mark.parametrize("where", ["host", "device"])
def test_stress_update_bit_exact(dims, per, where):
    """The projection-step stress update on the GPU against the numpy
    restatement of shear_sim_3d.cpp:681-710: the new stresses bit for bit,
    proj_mag (a sum over cells in another order) to 1e-13."""
    import stzpp_gb300 as sg
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    rng = np.random.default_rng(6)
    u = rng.standard_normal((m * n * o, 3))
    sig = P.random_strain(9, m, n, o, per)
    lam, mu, dt = 2.0, 1.0, 0.37
    want, modsq = P.stress_update(u, sig, lam, mu, dt, *h, dims, per)
    with sg.Multigrid(dims, per, precision="fp64") as mg:
        mg.set_x(u)
        if where == "host":
            got = np.ascontiguousarray(sig.copy())
            pm = mg.stress_update(got, lam, mu, dt, h)
        else:
            import torch
            t = torch.from_numpy(sig.copy()).cuda()
            pm = mg.stress_update(t, lam, mu, dt, h)
            got = t.cpu().numpy()
    assert np.array_equal(got, want)
    assert abs(pm - modsq.sum()) <= 1e-13 * modsq.sum()


def _proj_cases():
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "proj_step.npz"))
    for name in ("a", "b"):
        yield name, {k.split("/", 1)[1]: d[k] for k in d.files if k.startswith(name + "/")}


@pytest.mark.parametrize("where", ["host", "device"])
def test_rhs_and_stress_update_match_the_reference_step(where):
    """The GPU right-hand side assembly and stress update against the
    reference's own r_field and projection_step (tests/golden/proj_step.npz):
    the node right-hand side and the new stresses bit for bit from the same
    cell stresses and solved velocities, proj_mag to 1e-13 (another
    summation order)."""
    import stzpp_gb300 as sg
    for name, c in _proj_cases():
        nx, ny, nz = (int(v) for v in c["cells"])
        dims, per = (nx, ny, nz + 1), (True, True, False)
        h = P.grid_spacing(*dims, per)
        lamb, mu = (float(v) for v in c["lamb_mu"])
        with sg.Multigrid(dims, per, precision="fp64", max_coarse=10 ** 9) as mg:
            mg.set_rhs_divergence(np.ascontiguousarray(c["sigma"]), h)
            assert np.array_equal(mg.get_rhs(), c["rhs"]), name
            mg.set_x(np.ascontiguousarray(c["u"]))
            if where == "host":
                sig = np.ascontiguousarray(c["sigma"].copy())
                pm = mg.stress_update(sig, lamb, mu, float(c["dt"]), h)
            else:
                import torch
                t = torch.from_numpy(np.ascontiguousarray(c["sigma"].copy())).cuda()
                pm = mg.stress_update(t, lamb, mu, float(c["dt"]), h)
                sig = t.cpu().numpy()
        assert np.array_equal(sig, c["sigma_new"]), name
        assert abs(pm - float(c["proj_mag"])) <= 1e-13 * float(c["proj_mag"]), name
