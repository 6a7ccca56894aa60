"""The adjoint oracle (oracle/adjoint.py) on CPU: its coefficient gradient,
obtained by probing the operator's linearity in (mu, lam) with colour
classes, equals the node-by-node definition -w^T (A(e_q) u), and its total
gradient agrees with central finite differences of L(u(b, mu, lam))."""
import numpy as np
import pytest

from oracle import adjoint as AD
from oracle import problem as P

pytest.importorskip("scipy")

CASES = [((4, 4, 5), (True, True, False)), ((5, 4, 4), (False, True, False)), ((4, 5, 4), (True, False, True))]


def setup(dims, per, seed=2):
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    mu = P.lognormal_mu(seed, m, n, o)
    lam = 2 * mu * np.exp(0.1 * np.random.default_rng(seed + 1).standard_normal(mu.shape))
    rng = np.random.default_rng(seed + 2)
    b = rng.standard_normal((m * n * o, 3))
    ustar = rng.standard_normal((m * n * o, 3))
    return h, mu, lam, b, ustar


@pytest.mark.parametrize("dims,per", CASES)
def test_probing_equals_node_by_node_definition(dims, per):
    h, mu, lam, b, ustar = setup(dims, per)
    u, w, (gb, gmu, glam) = AD.gradients(mu, lam, h, per, b, lambda u: 2 * (u - ustar))
    N = mu.size
    nb = AD.neighbours(dims, per)
    ref_mu, ref_lam = np.zeros(N), np.zeros(N)
    for q in range(N):
        e = np.zeros(N)
        e[q] = 1.0
        e = e.reshape(mu.shape)
        ref_mu[q] = -(w * AD.apply_points(P.elastic_stencil_points(e, 0 * e, *h, per), u, nb)).sum()
        ref_lam[q] = -(w * AD.apply_points(P.elastic_stencil_points(0 * e, e, *h, per), u, nb)).sum()
    assert np.abs(gmu - ref_mu).max() <= 1e-13 * np.abs(ref_mu).max()
    assert np.abs(glam - ref_lam).max() <= 1e-13 * np.abs(ref_lam).max()


@pytest.mark.parametrize("dims,per", CASES)
def test_gradient_matches_central_differences(dims, per):
    h, mu, lam, b, ustar = setup(dims, per)
    m, n, o = dims
    u, w, (gb, gmu, glam) = AD.gradients(mu, lam, h, per, b, lambda u: 2 * (u - ustar))

    def L(mu_, lam_, b_):
        pts = P.elastic_stencil_points(mu_, lam_, *h, per)
        x = AD.solve(AD.assemble(pts, dims, per), b_)
        return ((x - ustar) ** 2).sum()

    rng = np.random.default_rng(9)
    eps = 1e-6
    fd, an = [], []
    for _ in range(4):
        dmu = rng.standard_normal(mu.shape) * mu
        dlam = rng.standard_normal(mu.shape) * lam
        db = rng.standard_normal(b.shape)
        fd.append((L(mu + eps * dmu, lam + eps * dlam, b + eps * db) -
                   L(mu - eps * dmu, lam - eps * dlam, b - eps * db)) / (2 * eps))
        an.append((gmu * dmu.ravel()).sum() + (glam * dlam.ravel()).sum() + (gb * db).sum())
    fd, an = np.array(fd), np.array(an)
    assert np.linalg.norm(fd - an) <= 1e-6 * np.linalg.norm(an)
