"""GPU adjoint of the projection solve, through the C-ABI and the autograd layer.

* stz_mg_adjoint_solve / stz_mg_coeff_grad against the adjoint oracle
  (oracle/adjoint.py: scipy direct solves of A and A^T, coefficient
  derivatives by linearity of the oracle's operator), FP64 and mixed, on
  multi-level hierarchies and all-Dirichlet / periodic mixes;
* the shared-stencil adjoint, including the Dirichlet nodes;
* the torch.autograd.Function at 128x128x129 (lognormal mu, sigma 0.3;
  L = |u - u*|^2, u* ~ N(0, 1e-3), seed 2): central finite differences with
  eps = 1e-6 along 32 random directions of (b, mu, lam), and the mixed
  gradient against the FP64 one;
* checkpointed sequences of solves give the gradient of the stored ones.
"""
import numpy as np
import pytest

from oracle import problem as P

pytestmark = pytest.mark.gpu

CASES = [((8, 8, 9), (True, True, False), 16),
         ((16, 16, 17), (True, True, False), 1024),
         ((16, 12, 10), (True, False, False), 32),
         ((10, 9, 8), (False, False, False), 64)]


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def problem(dims, per, seed=1):
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    mu = P.lognormal_mu(seed, m, n, o)
    lam = 2 * mu * np.exp(0.1 * np.random.default_rng(seed + 10).standard_normal(mu.shape))
    rng = np.random.default_rng(seed + 20)
    b = rng.standard_normal((m * n * o, 3))
    b[~P.interior_mask(m, n, o, *per).reshape(-1)] = 0.0
    ustar = rng.standard_normal((m * n * o, 3))
    return h, mu, lam, b, ustar


@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-12, 1e-8), ("mixed", 1e-10, 1e-6)])
@pytest.mark.parametrize("dims,per,mc", CASES)
def test_lame_adjoint_matches_oracle(dims, per, mc, precision, tol, bound):
    import stzpp_gb300 as sg
    from oracle import adjoint as AD
    h, mu, lam, b, ustar = problem(dims, per)
    u_o, w_o, (gb_o, gmu_o, glam_o) = AD.gradients(mu, lam, h, per, b, lambda u: 2 * (u - ustar))
    with sg.Multigrid(dims, per, precision=precision, max_coarse=mc) as mg:
        mg.setup_matrices(mu=mu.reshape(-1), lam=lam.reshape(-1), spacing=h)
        mg.setup_fields(r=b)
        mg.solve(tol, 200)
        u = mg.get_x()
        w, cycles, rr = mg.adjoint_solve(2 * (u - ustar), tol=tol, max_cycles=200)
        assert rr <= tol
        dmu, dlam = mg.coeff_grad(w, u)
    assert rel(u, u_o) <= bound
    assert rel(w, w_o) <= bound, rel(w, w_o)
    assert rel(dmu, gmu_o) <= bound, rel(dmu, gmu_o)
    assert rel(dlam, glam_o) <= bound, rel(dlam, glam_o)


def test_coeff_grad_exact_for_given_fields():
    """The contraction alone, on arbitrary w and u: no solve involved, so it
    must agree with the oracle's probing to FP64 round-off."""
    import stzpp_gb300 as sg
    from oracle import adjoint as AD
    for dims, per in (((8, 8, 9), (True, True, False)), ((7, 6, 5), (False, False, False)),
                      ((6, 8, 6), (True, False, True))):
        h, mu, lam, _, _ = problem(dims, per, seed=4)
        rng = np.random.default_rng(7)
        N = mu.size
        w, u = rng.standard_normal((N, 3)), rng.standard_normal((N, 3))
        gmu_o, glam_o = AD.coeff_grad(mu, lam, h, per, w, u)
        with sg.Multigrid(dims, per, precision="fp64", max_coarse=4096) as mg:
            mg.set_coeffs_lame(mu.reshape(-1), lam.reshape(-1), *h)
            dmu, dlam = mg.coeff_grad(w, u)
        assert np.abs(dmu - gmu_o).max() <= 1e-12 * np.abs(gmu_o).max()
        assert np.abs(dlam - glam_o).max() <= 1e-12 * np.abs(glam_o).max()


@pytest.mark.parametrize("dims,per", [((16, 16, 17), (True, True, False)), ((12, 10, 9), (False, False, False))])
def test_const_adjoint_with_dirichlet_nodes(dims, per):
    import stzpp_gb300 as sg
    from oracle import adjoint as AD
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
    g = np.random.default_rng(3).standard_normal((m * n * o, 3))   # non-zero on the plates too
    mu = np.ones((o, n, m))
    pts = P.elastic_stencil_points(mu, 2 * mu, *h, per)
    import scipy.sparse.linalg as spla
    w_o = spla.splu(AD.assemble(pts, dims, per).tocsc(), permc_spec="NATURAL").solve(g.reshape(-1), trans="T")
    with sg.Multigrid(dims, per, precision="fp64") as mg:
        mg.setup_matrices(*sg.elastic_stencil(1.0, 2.0, *h))
        w, cycles, rr = mg.adjoint_solve(g, tol=1e-12, max_cycles=200)
    assert rel(w, w_o.reshape(-1, 3)) <= 1e-8


# ------------------------------------------------------------ autograd
DIMS4 = (128, 128, 129)
PER4 = (True, True, False)


def config4_inputs():
    import torch
    m, n, o = DIMS4
    h = P.grid_spacing(m, n, o, PER4)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, PER4), m, n, o, PER4, *h)
    mu = P.lognormal_mu(1, m, n, o).reshape(-1)
    ustar = np.random.default_rng(2).normal(0.0, 1e-3, size=(m * n * o, 3))
    cuda = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return h, cuda(b), cuda(mu), cuda(2 * mu), cuda(ustar)


def grads(solver, b, mu, lam, ustar):
    import torch
    b, mu, lam = (t.detach().clone().requires_grad_(True) for t in (b, mu, lam))
    u = solver(b, mu, lam)
    L = ((u - ustar) ** 2).sum()
    L.backward()
    return float(L.detach()), b.grad, mu.grad, lam.grad


def test_autograd_central_differences_128():
    import torch
    from stzpp_gb300.autograd import ProjectionSolver
    h, b, mu, lam, ustar = config4_inputs()
    S = ProjectionSolver(DIMS4, PER4, h, precision="fp64", tol=1e-12, max_cycles=100)
    L0, gb, gmu, glam = grads(S, b, mu, lam, ustar)
    rng = np.random.default_rng(5)
    eps = 1e-6
    brms = float(b.pow(2).mean().sqrt())
    fd, an = [], []
    with torch.no_grad():
        for _ in range(32):
            db = torch.from_numpy(rng.standard_normal(tuple(b.shape)) * brms).cuda()
            dmu = torch.from_numpy(rng.standard_normal(tuple(mu.shape))).cuda() * mu
            dlam = torch.from_numpy(rng.standard_normal(tuple(lam.shape))).cuda() * lam
            up = S(b + eps * db, mu + eps * dmu, lam + eps * dlam)
            um = S(b - eps * db, mu - eps * dmu, lam - eps * dlam)
            # L(+) - L(-) = <u+ - u-, u+ + u- - 2 u*>: the same difference of
            # |u - u*|^2 without cancelling the large constant |u*|^2
            fd.append(float(((up - um) * (up + um - 2 * ustar)).sum()) / (2 * eps))
            an.append(float((gb * db).sum() + (gmu * dmu).sum() + (glam * dlam).sum()))
    fd, an = np.array(fd), np.array(an)
    err = np.linalg.norm(fd - an) / np.linalg.norm(an)
    print(f"128x128x129 adjoint vs central FD (eps 1e-6, 32 directions): rel L2 {err:.3e}, "
          f"max rel {np.max(np.abs(fd - an) / np.abs(an)):.3e}")
    assert err <= 1e-6
    S.close()


def test_autograd_mixed_vs_fp64_gradient_128():
    from stzpp_gb300.autograd import ProjectionSolver
    h, b, mu, lam, ustar = config4_inputs()
    out = {}
    for prec in ("fp64", "mixed"):
        S = ProjectionSolver(DIMS4, PER4, h, precision=prec, tol=1e-10 if prec == "mixed" else 1e-12)
        out[prec] = grads(S, b, mu, lam, ustar)
        S.close()
    errs = [rel(a.cpu().numpy(), r.cpu().numpy()) for a, r in zip(out["mixed"][1:], out["fp64"][1:])]
    print("mixed vs FP64 gradient (b, mu, lam):", ["%.2e" % e for e in errs])
    assert max(errs) <= 1e-6


def test_checkpointed_sequence_matches_stored():
    import torch
    from stzpp_gb300.autograd import ProjectionSolver, sequence_loss
    dims, per = (32, 32, 33), (True, True, False)
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    cuda = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    b0 = cuda(P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h))
    incs = [cuda(P.rhs_divergence(P.random_strain(100 + t, m, n, o, per, std=1e-5), m, n, o, per, *h))
            for t in range(6)]
    mu0 = cuda(P.lognormal_mu(1, m, n, o).reshape(-1))
    ustar = cuda(np.random.default_rng(3).normal(0, 1e-3, size=(m * n * o, 3)))
    res = {}
    for ck in (0, 2):
        S = ProjectionSolver(dims, per, h, precision="fp64", tol=1e-12)
        b = b0.clone().requires_grad_(True)
        mu = mu0.clone().requires_grad_(True)
        lam = (2 * mu0).clone().requires_grad_(True)
        L = sequence_loss(S, b, incs, mu, lam, lambda t, u: ((u - ustar) ** 2).sum(), checkpoint_every=ck)
        L.backward()
        res[ck] = (float(L), b.grad.cpu().numpy(), mu.grad.cpu().numpy(), lam.grad.cpu().numpy())
        S.close()
    assert abs(res[0][0] - res[2][0]) <= 1e-12 * abs(res[0][0])
    for a, c in zip(res[2][1:], res[0][1:]):
        assert rel(a, c) <= 1e-9


def test_forward_output_is_ready_on_torch_stream_256():
    """The solver works on its own stream; the tensor forward returns must be
    complete when torch's stream reads it straight away (256x256x257, so a
    missing synchronisation would show)."""
    import torch
    from stzpp_gb300.autograd import ProjectionSolver
    dims, per = (256, 256, 257), (True, True, False)
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    cuda = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    b = cuda(P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h))
    mu = torch.ones(m * n * o, dtype=torch.float64, device="cuda")
    lam = 2 * mu
    S = ProjectionSolver(dims, per, h, precision="mixed", tol=1e-8)
    u = S(b, mu, lam)
    early = u.clone()            # queued on torch's stream right after forward
    s1 = float(u.abs().sum())
    torch.cuda.synchronize()
    late = S.mg.get_x()          # the handle's solution, read back after a full synchronize
    S.close()
    assert np.array_equal(early.cpu().numpy(), late)
    assert s1 == float(np.abs(late).sum()) or abs(s1 - float(np.abs(late).sum())) <= 1e-12 * s1
