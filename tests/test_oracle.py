"""Pins the oracle (C restatement of the reference multigrid) to the reference.

* against the golden fixtures generated from the compiled reference
  (tests/golden/make_golden.py): box bounds bit-exact, coefficients, sweeps,
  transfers and V-cycle iterates to FP64 round-off;
* against the compiled reference itself (oracle/_ref) on more grids when it is
  available (built from the reference checkout on this machine);
* the operator and right-hand side definitions shared by the tests.
CPU only.
"""
import os

import numpy as np
import pytest

from oracle import problem as P

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_small.npz")
RTOL = 1e-12   # FP64 round-off after a few operations, max-norm relative


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


CASES = {"p110": ((8, 8, 9), (True, True, False), "const", 16),
         "d000": ((6, 5, 4), (False, False, False), "const", 8),
         "var": ((8, 8, 9), (True, True, False), "var", 16)}


def port_for(oracle_port, dims, per, kind, max_coarse):
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    if kind == "const":
        st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
        return oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=max_coarse)
    mu = P.lognormal_mu(1, m, n, o)
    return oracle_port.PortMultigrid(dims, per, points=P.elastic_stencil_points(mu, 2 * mu, *h, per),
                                     max_coarse=max_coarse)


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_golden(name, golden, oracle_port):
    dims, per, kind, mc = CASES[name]
    Q = port_for(oracle_port, dims, per, kind, mc)
    assert Q.nlevels == int(golden[f"{name}/nlevels"])
    for l in range(Q.nlevels):
        assert Q.level_dims(l) == tuple(golden[f"{name}/dims{l}"])
        assert np.array_equal(Q.level_S(l), golden[f"{name}/S{l}"].astype(np.int32)), f"S level {l}"
        if l > 0:
            assert rel(Q.level_A(l), golden[f"{name}/A{l}"]) < 1e-13, f"A level {l}"
    x0, b0 = golden[f"{name}/x0"], golden[f"{name}/b0"]
    Q.set_field(0, "x", x0)
    Q.set_field(0, "r", b0)
    Q.gauss_seidel(0, 1, smoother="lex")
    assert rel(Q.get_field(0, "x"), golden[f"{name}/gs0"]) < RTOL
    Q.restriction(1)
    assert rel(Q.get_field(1, "r"), golden[f"{name}/restrict1"]) < RTOL
    Q.set_field(1, "x", golden[f"{name}/xc1"])
    Q.interpolation(1)
    assert rel(Q.get_field(0, "x"), golden[f"{name}/interp0"]) < RTOL
    Q.set_field(0, "x", x0)
    Q.set_field(0, "r", b0)
    Q.v_cycle(bottom="gs", smoother="lex")
    Q.v_cycle(bottom="gs", smoother="lex")
    assert rel(Q.get_field(0, "x"), golden[f"{name}/vcycle2"]) < 1e-11


def test_port_matches_golden_solve(golden, oracle_port):
    """The 32x32x33 problem with the reference's own hierarchy and cycle."""
    m, n, o = 32, 32, 33
    per = (True, True, False)
    h = P.grid_spacing(m, n, o, per)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    assert abs(np.linalg.norm(b) - float(golden["cfg1/b_norm"])) <= 1e-15 * float(golden["cfg1/b_norm"])
    Q = port_for(oracle_port, (m, n, o), per, "const", 1024)
    Q.set_field(0, "r", b)
    Q.set_field(0, "x", np.zeros_like(b))
    cycles, hist = Q.solve(1e-10, 100, bottom="gs", smoother="lex")
    ref_hist = golden["cfg1/hist"]
    assert cycles == len(ref_hist)
    assert np.allclose(hist, ref_hist, rtol=1e-6, atol=0)
    x = Q.get_field(0, "x")
    assert rel(x[::97], golden["cfg1/x_sub"]) < 1e-9
    assert abs(np.linalg.norm(x) / float(golden["cfg1/x_norm"]) - 1) < 1e-10


# ---------------------------------------------------------------- live reference
REF_GRIDS = [((16, 16, 17), (True, True, False), "const", 16), ((12, 10, 9), (False, False, False), "const", 16),
             ((14, 12, 11), (True, False, False), "const", 16), ((9, 7, 8), (False, True, False), "const", 8),
             ((13, 11, 9), (False, False, True), "const", 8), ((16, 16, 17), (True, True, False), "var", 16),
             ((32, 32, 33), (True, True, False), "const", 1024)]


@pytest.mark.parametrize("dims,per,kind,mc", REF_GRIDS)
def test_port_matches_live_reference(dims, per, kind, mc, oracle_port):
    from oracle import refpy
    if not refpy.available():
        pytest.skip("compiled reference not available on this machine")
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    if kind == "const":
        st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
        kw = dict(stencil=st, fix=fix)
    else:
        mu = P.lognormal_mu(1, m, n, o)
        kw = dict(points=P.elastic_stencil_points(mu, 2 * mu, *h, per))
    R = refpy.RefMultigrid(dims, per, max_coarse=mc, **kw)
    Q = oracle_port.PortMultigrid(dims, per, max_coarse=mc, **kw)
    assert R.nlevels == Q.nlevels
    rng = np.random.default_rng(5)
    for l in range(R.nlevels):
        assert R.level_dims(l) == Q.level_dims(l)
        assert np.array_equal(R.level_S(l), Q.level_S(l))
        assert rel(Q.level_A(l), R.level_A(l)) < 1e-13
        N = R.npts(l)
        x, b = rng.standard_normal((N, 3)), rng.standard_normal((N, 3))
        for M in (R, Q):
            M.set_field(l, "x", x)
            M.set_field(l, "r", b)
        R.gauss_seidel(l, 1)
        Q.gauss_seidel(l, 1, smoother="lex")
        assert rel(Q.get_field(l, "x"), R.get_field(l, "x")) < RTOL
        assert rel(Q.residual(l)[0], R.residual(l)[0]) < RTOL
        if l + 1 < R.nlevels:
            R.restriction(l + 1)
            Q.restriction(l + 1)
            assert rel(Q.get_field(l + 1, "r"), R.get_field(l + 1, "r")) < RTOL
            xc = rng.standard_normal((R.npts(l + 1), 3))
            R.set_field(l + 1, "x", xc)
            Q.set_field(l + 1, "x", xc)
            R.interpolation(l + 1)
            Q.interpolation(l + 1)
            assert rel(Q.get_field(l, "x"), R.get_field(l, "x")) < RTOL
    x0 = rng.standard_normal((R.npts(0), 3))
    b0 = rng.standard_normal((R.npts(0), 3))
    for M in (R, Q):
        M.set_field(0, "x", x0)
        M.set_field(0, "r", b0)
    for _ in range(2):
        R.v_cycle("gs")
        Q.v_cycle(bottom="gs", smoother="lex")
    assert rel(Q.get_field(0, "x"), R.get_field(0, "x")) < 1e-11


def test_reference_l2_error_all_is_sum_of_fourth_powers(oracle_port):
    """Quirk: region::l2_error_all for V=vec3 sums |r|^4 (mg3d_mod_sq of the vec3->double cast)."""
    from oracle import refpy
    if not refpy.available():
        pytest.skip("compiled reference not available on this machine")
    dims, per = (8, 8, 9), (True, True, False)
    h = P.grid_spacing(*dims, per)
    st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
    R = refpy.RefMultigrid(dims, per, stencil=st, fix=fix)
    rng = np.random.default_rng(2)
    R.set_field(0, "x", rng.standard_normal((R.npts(0), 3)))
    R.set_field(0, "r", rng.standard_normal((R.npts(0), 3)))
    r, _ = R.residual(0)
    q = (r * r).sum(axis=1)
    assert abs(R.l2_error_all(0) - (q * q).sum()) <= 1e-12 * (q * q).sum()


# ---------------------------------------------------------------- problem
def test_product_stencil_matches_oracle_stencil():
    import stzpp_gb300 as sg
    for h in ((1 / 32, 1 / 32, 1 / 32), (0.1, 0.2, 0.05)):
        a, fa = sg.elastic_stencil(1.3, 2.1, *h, dt=0.7)
        b, fb = P.elastic_stencil_const(1.3, 2.1, *h, dt=0.7)
        assert np.allclose(a, b, rtol=1e-15, atol=0) and np.allclose(fa, fb, rtol=1e-15, atol=0)


def test_variable_operator_reduces_to_constant_stencil():
    dims, per = (6, 6, 7), (True, True, False)
    h = P.grid_spacing(*dims, per)
    mu = np.full((7, 6, 6), 1.0)
    pts = P.elastic_stencil_points(mu, 2 * mu, *h, per).reshape(7, 6, 6, 27, 9)
    st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
    assert np.allclose(pts[3, 2, 2], st, rtol=1e-14, atol=0)
    assert np.allclose(pts[0, 1, 1, 13], fix, rtol=1e-14, atol=0)
    assert not pts[0, 1, 1, :13].any() and not pts[0, 1, 1, 14:].any()


def test_variable_operator_is_symmetric_on_the_interior():
    """A[p, p+d] = A[p+d, p]^T between interior nodes (the discretisation is
    the Galerkin form of a symmetric bilinear form)."""
    dims, per = (6, 6, 7), (True, True, False)
    h = P.grid_spacing(*dims, per)
    mu = P.lognormal_mu(4, *dims)
    pts = P.elastic_stencil_points(mu, 2 * mu, *h, per).reshape(7, 6, 6, 27, 3, 3)
    for k in range(2, 5):
        for j in range(6):
            for i in range(6):
                for dz in (-1, 0, 1):
                    for dy in (-1, 0, 1):
                        for dx in (-1, 0, 1):
                            b = P.block_index(dx, dy, dz)
                            q = (k + dz, (j + dy) % 6, (i + dx) % 6)
                            bt = P.block_index(-dx, -dy, -dz)
                            assert np.allclose(pts[k, j, i, b], pts[q][bt].T, rtol=1e-13, atol=1e-9)


def test_rhs_vanishes_on_dirichlet_nodes_and_sums_to_zero_in_periodic_dims():
    dims, per = (8, 8, 9), (True, True, False)
    h = P.grid_spacing(*dims, per)
    b = P.rhs_divergence(P.random_strain(0, *dims, per), *dims, per, *h).reshape(9, 8, 8, 3)
    assert not b[0].any() and not b[-1].any()
    # the x-derivative terms telescope over a periodic x-row
    assert np.isfinite(b).all() and np.abs(b).max() > 0


# ---------------------------------------------------------------- trans_sim frames
TRANS = os.path.join(HERE, "golden", "trans_stencils.npz")


def test_trans_fixture_matches_reference_functions():
    """The golden transformed-frame stencils are what the reference's
    generated functions give (oracle/trans_stencil.py harness), and the
    identity frame is the shear_sim elasticity stencil."""
    import ctypes
    d = np.load(TRANS)
    lib_path = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libtransstencil.so")
    if os.path.exists(lib_path):
        lib = ctypes.CDLL(lib_path)
        lib.ref_trans_stencil.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 6 + [ctypes.c_void_p] * 2
        for c in range(len(d["T"])):
            t = np.ascontiguousarray(d["T"][c])
            S, F = np.zeros(243), np.zeros(9)
            lib.ref_trans_stencil(t.ctypes.data_as(ctypes.c_void_p), 1.0, 2.0, 1.0, 1.0, 1.0, 1.0,
                                  S.ctypes.data_as(ctypes.c_void_p), F.ctypes.data_as(ctypes.c_void_p))
            assert np.array_equal(S, d["stencil"][c]) and np.array_equal(F, d["fix"][c])
        t = np.ascontiguousarray(np.eye(3))
        S, F = np.zeros(243), np.zeros(9)
        lib.ref_trans_stencil(t.ctypes.data_as(ctypes.c_void_p), 1.0, 2.0, 1.0, 1.0, 1.0, 1.0,
                              S.ctypes.data_as(ctypes.c_void_p), F.ctypes.data_as(ctypes.c_void_p))
        st, fix = P.elastic_stencil_const(1.0, 2.0, 1.0, 1.0, 1.0)
        assert np.array_equal(S.reshape(27, 9), st) and np.array_equal(F, fix)
    S = d["stencil"].reshape(-1, 27, 3, 3)
    assert not any(np.allclose(S[c], np.swapaxes(S[c][::-1], 1, 2)) for c in range(len(S)))   # non-symmetric


@pytest.mark.parametrize("frame", [0, 1, 2])
def test_port_matches_live_reference_trans(frame, oracle_port):
    """The C restatement against the compiled reference on a transformed-frame
    (full, non-symmetric) shared stencil: coarse operators, sweeps, transfers
    and V-cycles."""
    from oracle import refpy
    if not refpy.available():
        pytest.skip("compiled reference not available on this machine")
    dims, per = (16, 16, 17), (True, True, False)
    h = 1.0 / 16
    d = np.load(TRANS)
    st, fix = d["stencil"][frame].reshape(27, 9) / (h * h), d["fix"][frame] / (h * h)
    R = refpy.RefMultigrid(dims, per, stencil=st, fix=fix, max_coarse=16)
    Q = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=16)
    assert R.nlevels == Q.nlevels
    rng = np.random.default_rng(frame)
    for l in range(R.nlevels):
        assert np.array_equal(R.level_S(l), Q.level_S(l))
        assert rel(Q.level_A(l), R.level_A(l)) < 1e-13
    x0 = rng.standard_normal((R.npts(0), 3))
    b0 = rng.standard_normal((R.npts(0), 3))
    for M in (R, Q):
        M.set_field(0, "x", x0)
        M.set_field(0, "r", b0)
    for _ in range(2):
        R.v_cycle("gs")
        Q.v_cycle(bottom="gs", smoother="lex")
    assert rel(Q.get_field(0, "x"), R.get_field(0, "x")) < 1e-11


def test_threaded_port_matches_serial(oracle_port):
    """The oracle on several threads (the reference's sweep on z-slab
    sub-domains with ghosts refreshed once per sweep, as on MPI ranks split
    along z): single transfers and residuals equal the serial ones to
    round-off, and the converged solution is the serial one."""
    dims, per = (32, 32, 33), (True, True, False)
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    x0 = np.random.default_rng(4).standard_normal(b.shape) * 1e-4
    out = {}
    try:
        for T in (1, 4):
            assert oracle_port.set_threads(T) in (1, T)
            Q = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix)
            Q.set_field(0, "r", b)
            Q.set_field(0, "x", x0)
            res, sq = Q.residual(0)
            Q.restriction(1)
            r1 = Q.get_field(1, "r")
            Q.set_field(1, "x", r1)
            Q.interpolation(1)
            xi = Q.get_field(0, "x")
            Q.set_field(0, "x", np.zeros_like(b))
            cycles, _ = Q.solve(1e-12, 100)
            out[T] = (res, sq, r1, xi, Q.get_field(0, "x"), [Q.level_A(l) for l in range(Q.nlevels)])
    finally:
        oracle_port.set_threads(1)
    s, t = out[1], out[4]
    assert np.array_equal(s[0], t[0]) and abs(s[1] - t[1]) <= 1e-13 * s[1]
    assert np.abs(s[2] - t[2]).max() <= 1e-14 * np.abs(s[2]).max()
    assert np.abs(s[3] - t[3]).max() <= 1e-14 * np.abs(s[3]).max()
    assert rel(t[4], s[4]) <= 1e-9
    for a, c in zip(s[5], t[5]):
        assert np.abs(a - c).max() <= 1e-13 * np.abs(a).max()
