"""The C restatement of the quasi-static advection step (oracle/stzadv_oracle.c)
against the unmodified reference step (shear_sim_3d::advection_step,
src/shear_sim_3d.cpp:393-525): bit for bit against the golden fixture made
from the reference (tests/golden/adv_step.npz), and against the reference
itself where oracle/_ref/libstzadv.so was built (`make -C oracle advref`)."""
import os

import numpy as np
import pytest

from oracle import advect as A
from oracle import problem as P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "adv_step.npz")
ADV_IN = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 19, 27]
ADV_OUT = [13, 14, 15, 16, 17, 18, 19, 26, 27]
CASES = ["elastic", "mixed", "plastic", "long"]


def golden_case(name):
    """(fields, dims, params, dt, expected changed members) of a fixture case."""
    d = np.load(GOLD)
    nx, ny, nz = (int(v) for v in d[name + "/dims"])
    F = np.zeros((d[name + "/in"].shape[0], A.NFIELD))
    F[:, ADV_IN] = d[name + "/in"]
    prm = dict(zip(A.PARAM_NAMES, d[name + "/params"]))
    return F, (nx, ny, nz), prm, float(d[name + "/dt"]), d[name + "/out"]


@pytest.mark.parametrize("name", CASES)
def test_restatement_matches_reference_fixture(name):
    F, (nx, ny, nz), prm, dt, expect = golden_case(name)
    P, yielded = A.port_step(F, nx, ny, nz, prm, dt)
    assert np.array_equal(P[:, ADV_OUT], expect)
    others = [c for c in range(A.NFIELD) if c not in ADV_OUT]
    assert np.array_equal(P[:, others], F[:, others])
    assert yielded == (name != "elastic")


def test_fixture_exercises_both_regimes():
    for name in CASES:
        F, (nx, ny, nz), prm, dt, expect = golden_case(name)
        adpl = A.interior(expect[:, -1], nx, ny, nz)
        plastic = int((adpl > 0).sum())
        assert (plastic == 0) if name == "elastic" else (0 < plastic < nx * ny * nz)


@pytest.mark.skipif(not A.reference_available(), reason="oracle/_ref/libstzadv.so not built (no reference checkout)")
@pytest.mark.parametrize("dims,seed,dt,bias", [((12, 10, 8), 5, 800.0, 0.3), ((9, 7, 6), 6, 100.0, 1.0),
                                               ((4, 4, 3), 7, 3000.0, 0.8)])
def test_restatement_matches_live_reference(dims, seed, dt, bias):
    nx, ny, nz = dims
    prm = A.driver_params(nx)
    F = A.random_fields(seed, nx, ny, nz, plastic_bias=bias)
    R = A.reference_step(F, nx, ny, nz, prm, dt)
    P, _ = A.port_step(F, nx, ny, nz, prm, dt)
    assert np.array_equal(R, P)


# ------------------------------------------- the steps on either side of the solve
def _proj_cases():
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "proj_step.npz"))
    for name in ("a", "b"):
        yield name, {k.split("/", 1)[1]: d[k] for k in d.files if k.startswith(name + "/")}


def test_rhs_and_stress_update_restatements_match_the_reference_fixture():
    """The numpy restatements of r_field (the node divergence of the cell
    stresses) and of the projection-step stress update equal, bit for bit,
    the reference's own r_field and projection_step (tests/golden/proj_step.npz,
    made by tests/golden/make_golden.py proj from the compiled reference)."""
    for name, c in _proj_cases():
        nx, ny, nz = (int(v) for v in c["cells"])
        dims, per = (nx, ny, nz + 1), (True, True, False)
        h = P.grid_spacing(*dims, per)
        assert np.array_equal(P.rhs_divergence(c["sigma"], *dims, per, *h), c["rhs"]), name
        lamb, mu = c["lamb_mu"]
        new, modsq = P.stress_update(c["u"], c["sigma"], lamb, mu, float(c["dt"]), *h, dims, per)
        assert np.array_equal(new, c["sigma_new"]), name
        assert abs(modsq.sum() - float(c["proj_mag"])) <= 1e-13 * float(c["proj_mag"])


def test_projection_step_live_against_the_reference():
    """Where the reference is compiled: its r_field and projection step on a
    grid the fixture does not hold, against the restatements."""
    from oracle import advect as A
    if not A.reference_available():
        pytest.skip("compiled reference not available on this machine")
    nx, ny, nz = 10, 8, 6
    prm = A.driver_params(nx)
    F = A.random_fields(13, nx, ny, nz, sigma_scale=0.4)
    dims, per = (nx, ny, nz + 1), (True, True, False)
    h = P.grid_spacing(*dims, per)
    sig = A.cell_stresses(F, nx, ny, nz)
    assert np.array_equal(A.reference_rhs(F, nx, ny, nz, prm), P.rhs_divergence(sig, *dims, per, *h))
    G, pm = A.reference_projection(F, nx, ny, nz, prm, 0.005)
    new, modsq = P.stress_update(A.node_velocities(G, nx, ny, nz), sig, prm["lamb"], prm["mu"], 0.005, *h, dims, per)
    assert np.array_equal(new, A.cell_stresses(G, nx, ny, nz))
    assert abs(modsq.sum() - pm) <= 1e-13 * pm
