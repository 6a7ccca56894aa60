"""The GPU quasi-static advection step (stz_mg_advection_step) against the
reference: the golden fixture made from the unmodified reference step and the
C restatement pinned to it (oracle/stzadv_oracle.c).

Where no point reaches the yield stress the step uses no transcendental
function and must equal the reference bit for bit.  Above it, the STZ plastic
rate goes through exp (CUDA's on the GPU, the C library's on the host, which
may differ in the last bit), so those results are compared within a relative
tolerance of 1e-10 of each member's magnitude."""
import numpy as np
import pytest

from oracle import advect as A
from test_oracle_advect import ADV_OUT, CASES, golden_case

pytestmark = pytest.mark.gpu

TOL = 1e-10
MEMBERS = {"u": A.U, "v": A.V, "w": A.W, "s11": A.S11, "s12": A.S12, "s13": A.S13, "s22": A.S22, "s23": A.S23,
           "s33": A.S33, "chi": A.CHI, "ad_dpl": A.ADPL, "sbar": A.SBAR, "cs11": A.CS11, "cs12": A.CS12,
           "cs13": A.CS13, "cs22": A.CS22, "cs23": A.CS23, "cs33": A.CS33, "cchi": A.CCHI}


def gpu_step(F, dims, prm, dt):
    """One GPU step on the Field array F (npoints, 28); returns (new F, yielded)."""
    import torch
    from stzpp_gb300 import advect
    nx, ny, nz = dims
    fields = {k: torch.tensor(np.ascontiguousarray(F[:, c]), dtype=torch.float64, device="cuda")
              for k, c in MEMBERS.items()}
    yielded = advect.advection_step(fields, dims, (1.0 / nx, 1.0 / ny, 1.0 / nz), prm, dt)
    G = F.copy()
    for k, c in MEMBERS.items():
        G[:, c] = fields[k].cpu().numpy()
    return G, yielded


def rel_err(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


def test_elastic_step_is_the_reference_bit_for_bit():
    F, dims, prm, dt, expect = golden_case("elastic")
    G, yielded = gpu_step(F, dims, prm, dt)
    assert not yielded
    assert np.array_equal(G[:, ADV_OUT], expect)


@pytest.mark.parametrize("name", [c for c in CASES if c != "elastic"])
def test_plastic_steps_match_the_reference(name):
    F, dims, prm, dt, expect = golden_case(name)
    G, yielded = gpu_step(F, dims, prm, dt)
    assert yielded
    for j, c in enumerate(ADV_OUT):
        assert rel_err(G[:, c], expect[:, j]) <= TOL, f"member {c}: {rel_err(G[:, c], expect[:, j]):.3e}"
    others = [c for c in range(A.NFIELD) if c not in ADV_OUT]
    assert np.array_equal(G[:, others], F[:, others])


@pytest.mark.parametrize("dims,seed,dt,bias,sigma", [((48, 40, 24), 11, 500.0, 0.0, 0.7),
                                                     ((64, 32, 16), 12, 500.0, 0.0, 0.2),
                                                     ((33, 17, 9), 13, 1500.0, 0.9, 0.7),
                                                     ((1, 1, 1), 14, 100.0, 1.0, 0.7)])
def test_matches_the_restatement(dims, seed, dt, bias, sigma):
    """Larger, odd and single-cell grids against the C restatement (bitwise
    where nothing yields)."""
    nx, ny, nz = dims
    prm = A.driver_params(nx)
    F = A.random_fields(seed, nx, ny, nz, sigma_scale=sigma, plastic_bias=bias)
    P, py = A.port_step(F, nx, ny, nz, prm, dt)
    G, gy = gpu_step(F, dims, prm, dt)
    assert gy == py
    if not py:
        assert np.array_equal(G, P)
    else:
        for c in ADV_OUT:
            assert rel_err(G[:, c], P[:, c]) <= TOL, f"member {c}: {rel_err(G[:, c], P[:, c]):.3e}"


def test_rejects_bad_arguments():
    import torch
    from stzpp_gb300 import advect, mg
    dims = (4, 4, 4)
    n = advect.grid_points(*dims)
    fields = {k: torch.zeros(n, dtype=torch.float64, device="cuda") for k in advect.INPUTS + advect.OUTPUTS}
    prm = A.driver_params(4)
    with pytest.raises(mg.StzMgError):
        advect.advection_step(fields, dims, (0.25,) * 3, prm, 0.0)
    with pytest.raises(ValueError):
        advect.advection_step(dict(fields, chi=torch.zeros(n - 1, dtype=torch.float64, device="cuda")), dims,
                              (0.25,) * 3, prm, 1.0)
