"""The C restatement of the quasi-static advection step (oracle/stzadv_oracle.c)
against the unmodified reference step (shear_sim_3d::advection_step,
src/shear_sim_3d.cpp:393-525): bit for bit against the golden fixture made
from the reference (tests/golden/adv_step.npz), and against the reference
itself where oracle/_ref/libstzadv.so was built (`make -C oracle advref`)."""
import os

import numpy as np
import pytest

from oracle import advect as A

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
