"""GPU parity: the CUDA path through the C-ABI against the oracle.

The oracle is the C restatement of the reference multigrid (oracle/), itself
pinned to the compiled reference by tests/test_oracle.py and the golden
fixtures.  Kernels are compared one by one on the same seeded inputs (box
bounds exactly; coefficients, sweeps and transfers to FP64 round-off), then
whole V-cycles with the same smoother order, then converged solutions against
the reference's own lexicographic solver (relative L2 error <= 1e-9).
"""
import numpy as np
import pytest

from oracle import problem as P

pytestmark = pytest.mark.gpu

# round-off tolerance for one kernel in FP64: max-norm error relative to the
# max-norm of the oracle's output
KERNEL_RTOL = 1e-13
# converged-solution tolerance of the projection solve (relative L2)
SOLUTION_RTOL = 1e-9

GRIDS = [
    ((16, 16, 17), (True, True, False), "const"),
    ((16, 16, 17), (True, True, False), "trans"),
    ((16, 16, 17), (True, True, False), "points"),
    ((16, 16, 17), (True, True, False), "lame"),
    ((12, 10, 9), (False, False, False), "const"),
    ((16, 12, 10), (True, False, False), "const"),
]


def trans_stencil(c, h):
    """Frame c of the reference's transformed-frame stencils (trans_sim_3d,
    golden fixture computed at dx = dy = dz = 1) on a grid of spacing h: a
    full, non-symmetric shared stencil (the coefficient-change path)."""
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "trans_stencils.npz"))
    return d["stencil"][c].reshape(27, 9) / (h * h), d["fix"][c] / (h * h)


def rel_max(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def build_pair(dims, per, kind, oracle_port, max_coarse=16, precision="fp64", bottom="direct"):
    import stzpp_gb300 as sg
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per)
    mg = sg.Multigrid(dims, per, precision=precision, max_coarse=max_coarse, bottom=bottom)
    if kind == "const":
        st, fix = P.elastic_stencil_const(1.0, 2.0, dx, dy, dz)
        ref = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=max_coarse)
        st_gpu, fix_gpu = sg.elastic_stencil(1.0, 2.0, dx, dy, dz)
        mg.setup_matrices(stencil=st_gpu, fix=fix_gpu)
    elif kind == "trans":
        st, fix = trans_stencil(0, dx)
        ref = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=max_coarse)
        mg.setup_matrices(stencil=st, fix=fix)
    else:
        mu = P.lognormal_mu(1, m, n, o)
        pts = P.elastic_stencil_points(mu, 2 * mu, dx, dy, dz, per)
        ref = oracle_port.PortMultigrid(dims, per, points=pts, max_coarse=max_coarse)
        if kind == "points":
            mg.setup_matrices(points=pts)
        else:
            mg.setup_matrices(mu=mu.reshape(-1), lam=(2 * mu).reshape(-1), spacing=(dx, dy, dz))
    return mg, ref


@pytest.mark.parametrize("dims,per,kind", GRIDS)
def test_hierarchy_and_operators(dims, per, kind, oracle_port):
    mg, ref = build_pair(dims, per, kind, oracle_port)
    assert mg.nlevels == ref.nlevels
    for l in range(mg.nlevels):
        assert mg.level_dims(l) == ref.level_dims(l)
        A, S = mg.level_operator(l)
        assert np.array_equal(S, ref.level_S(l)), f"box bounds differ on level {l}"
        Ar = ref.level_A(l)
        assert rel_max(A, Ar) < KERNEL_RTOL, f"level {l} coefficients: {rel_max(A, Ar):.3e}"
    mg.close()


@pytest.mark.parametrize("dims,per,kind", GRIDS)
def test_level_kernels(dims, per, kind, oracle_port):
    mg, ref = build_pair(dims, per, kind, oracle_port)
    rng = np.random.default_rng(7)
    for l in range(mg.nlevels):
        N = mg.level_npts(l)
        x = rng.standard_normal((N, 3))
        r = rng.standard_normal((N, 3))
        for M in (mg,):
            M.level_set_field(l, "x", x)
            M.level_set_field(l, "r", r)
        ref.set_field(l, "x", x)
        ref.set_field(l, "r", r)
        # residual
        res_g, sq_g = mg.residual(l)
        res_o, sq_o = ref.residual(l)
        assert rel_max(res_g, res_o) < KERNEL_RTOL
        assert abs(sq_g - sq_o) <= 1e-12 * sq_o
        # one 8-colour sweep
        mg.gauss_seidel(l, 1)
        ref.gauss_seidel(l, 1, smoother="mc8")
        assert rel_max(mg.level_get_field(l, "x"), ref.get_field(l, "x")) < KERNEL_RTOL
        if l + 1 < mg.nlevels:
            mg.restriction(l + 1)
            ref.restriction(l + 1)
            assert rel_max(mg.level_get_field(l + 1, "r"), ref.get_field(l + 1, "r")) < KERNEL_RTOL
            assert not mg.level_get_field(l + 1, "x").any()
            xc = rng.standard_normal((mg.level_npts(l + 1), 3))
            mg.level_set_field(l + 1, "x", xc)
            ref.set_field(l + 1, "x", xc)
            mg.interpolation(l + 1)
            ref.interpolation(l + 1)
            assert rel_max(mg.level_get_field(l, "x"), ref.get_field(l, "x")) < KERNEL_RTOL
    mg.close()


@pytest.mark.parametrize("dims,per,kind", GRIDS[:4])
def test_vcycle_iterates(dims, per, kind, oracle_port):
    """Whole V-cycles: same smoother order (8 colours), same direct bottom."""
    mg, ref = build_pair(dims, per, kind, oracle_port)
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, dx, dy, dz)
    mg.setup_fields(r=b)
    ref.set_field(0, "r", b)
    ref.set_field(0, "x", np.zeros_like(b))
    for c in range(3):
        mg.v_cycle()
        ref.v_cycle(bottom="direct", smoother="mc8")
        xg, xo = mg.get_x(), ref.get_field(0, "x")
        assert rel_max(xg, xo) < 1e-11, f"cycle {c}: {rel_max(xg, xo):.3e}"
    mg.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["const", "lame", "trans"])
def test_solution_matches_reference_solver(precision, kind, oracle_port):
    """32x32x33 (dx = 1/32), periodic x,y, Dirichlet z: converged solution of the
    GPU solve against the reference's lexicographic solver with its own
    hierarchy (coarsest level <= 1024 nodes, 24 GS sweeps at the bottom)."""
    import stzpp_gb300 as sg
    dims, per = (32, 32, 33), (True, True, False)
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, dx, dy, dz)
    if kind == "const":
        st, fix = P.elastic_stencil_const(1.0, 2.0, dx, dy, dz)
        ref = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=1024)
    elif kind == "trans":
        st, fix = trans_stencil(2, dx)
        ref = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=1024)
    else:
        mu = P.lognormal_mu(1, m, n, o)
        ref = oracle_port.PortMultigrid(dims, per, points=P.elastic_stencil_points(mu, 2 * mu, dx, dy, dz, per),
                                        max_coarse=1024)
    ref.set_field(0, "r", b)
    ref.set_field(0, "x", np.zeros_like(b))
    cyc_ref, hist = ref.solve(1e-13, 200, bottom="gs", smoother="lex")
    x_ref = ref.get_field(0, "x")
    with sg.Multigrid(dims, per, precision=precision) as mg:
        if kind == "const":
            mg.setup_matrices(*sg.elastic_stencil(1.0, 2.0, dx, dy, dz))
        elif kind == "trans":
            mg.setup_matrices(stencil=st, fix=fix)
        else:
            mg.setup_matrices(mu=mu.reshape(-1), lam=(2 * mu).reshape(-1), spacing=(dx, dy, dz))
        mg.setup_fields(r=b)
        cycles, rel = mg.solve(1e-10, 100)
        x = mg.get_x()
        rn, bn = mg.residual_norm()
    assert rel <= 1e-10 and rn / bn <= 1e-10
    err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    assert err <= SOLUTION_RTOL, f"{precision}/{kind}: {cycles} cycles, error {err:.3e}"


@pytest.mark.parametrize("pairs", ["1", "0"])
@pytest.mark.parametrize("kind", ["const", "const_inexact", "trans"])
def test_double_float_residual_matches_fp64(kind, pairs, monkeypatch):
    """The mixed solver's top-level residual in double-float arithmetic (FP32
    pairs, exact products, compensated sums; for the elastic stencils, whose
    blocks d and -d are equal, one product per pair of opposite neighbours
    unless STZ_MG_DF_PAIRS=0): after 3, 6, 9 and 12 cycles the
    relative residual it reports equals the FP64 residual norm of the same x
    to 1e-3 of itself plus 1e-13, and a solve with the FP64 residual kernel
    (STZ_MG_DF=0) takes the same number of cycles to a solution within 1e-10
    of it (both stop at a relative residual near 1e-10).  64x64x65,
    dx = 1/64: a full non-symmetric shared stencil, and the elastic one with
    mu = 1, lambda = 2 (every coefficient exact in FP32: the kernel without
    low coefficient halves) and with mu = 1.1, lambda = 2.3 (with them)."""
    import stzpp_gb300 as sg
    dims, per = (64, 64, 65), (True, True, False)
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, dx, dy, dz)
    if kind == "trans":
        st, fix = trans_stencil(2, dx)
    else:
        st, fix = sg.elastic_stencil(*((1.0, 2.0) if kind == "const" else (1.1, 2.3)), dx, dy, dz)
    monkeypatch.setenv("STZ_MG_DF_PAIRS", pairs)
    for cap in (3, 6, 9, 12):
        with sg.Multigrid(dims, per, precision="mixed") as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            mg.setup_fields(r=b)
            cycles, rel = mg.solve(1e-14, cap, check=False)
            rn, bn = mg.residual_norm()
        assert cycles == cap
        assert abs(rel - rn / bn) <= 1e-3 * (rn / bn) + 1e-13, f"{cap} cycles: {rel:.6e} vs FP64 {rn / bn:.6e}"
    out = {}
    for df in ("1", "0"):
        monkeypatch.setenv("STZ_MG_DF", df)
        with sg.Multigrid(dims, per, precision="mixed") as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            mg.setup_fields(r=b)
            out[df] = mg.solve(1e-10, 100) + (mg.get_x(),)
    assert out["1"][0] == out["0"][0]
    assert out["1"][1] <= 1e-10 and out["0"][1] <= 1e-10
    assert np.linalg.norm(out["1"][2] - out["0"][2]) <= 1e-10 * np.linalg.norm(out["0"][2])


def test_reference_hierarchy_gs_bottom(oracle_port):
    """The reference's own cycle shape (coarsest <= 1024 nodes, 24 GS sweeps)."""
    mg, ref = build_pair((32, 32, 33), (True, True, False), "const", oracle_port, max_coarse=1024, bottom="gs")
    assert mg.nlevels == ref.nlevels == 3
    m, n, o = 32, 32, 33
    dx, dy, dz = P.grid_spacing(m, n, o, (True, True, False))
    b = P.rhs_divergence(P.random_strain(0, m, n, o, (True, True, False)), m, n, o, (True, True, False), dx, dy, dz)
    mg.setup_fields(r=b)
    ref.set_field(0, "r", b)
    ref.set_field(0, "x", np.zeros_like(b))
    for c in range(2):
        mg.v_cycle()
        ref.v_cycle(bottom="gs", smoother="mc8")
    assert rel_max(mg.get_x(), ref.get_field(0, "x")) < 1e-11
    mg.close()



TILE_LEVEL_CASES = [((64, 64, 17), (True, True, False), "const", 0, 2), ((64, 64, 16), (True, True, True), "const", 0, 2),
                    ((96, 64, 9), (True, True, False), "const", 0, 4), ((128, 128, 17), (True, True, False), "const", 1, 2),
                    ((128, 128, 16), (True, True, True), "const", 1, 3), ((64, 64, 17), (True, True, False), "trans", 0, 2),
                    ((64, 64, 16), (True, True, True), "trans", 0, 3), ((128, 128, 17), (True, True, False), "trans", 1, 2)]


@pytest.mark.parametrize("dims,per,kind,level,sweeps", TILE_LEVEL_CASES)
def test_tiled_sweep_is_the_colour_sweep(dims, per, kind, level, sweeps, monkeypatch):
    """The tiled two-buffer sweep (each CTA runs a plane tile's four colours
    from shared memory, recomputing a 4-node halo) gives bit-for-bit the
    result of the eight colour launches: FP64 level sweeps of the elastic and
    of a full non-symmetric shared stencil and of their plane-invariant
    coarse operators, Dirichlet and periodic z, even and odd sweep counts."""
    import stzpp_gb300 as sg
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per)
    st, fix = sg.elastic_stencil(1.0, 2.0, dx, dy, dz) if kind == "const" else trans_stencil(2, dx)
    out = {}
    for tile in ("0", "1"):
        monkeypatch.setenv("STZ_MG_TILE", tile)
        with sg.Multigrid(dims, per, precision="fp64", bottom="gs", max_coarse=5000) as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            N = mg.level_npts(level)
            rng = np.random.default_rng(8)
            mg.level_set_field(level, "x", rng.standard_normal((N, 3)))
            mg.level_set_field(level, "r", rng.standard_normal((N, 3)))
            mg.gauss_seidel(level, sweeps)
            out[tile] = mg.level_get_field(level, "x")
    assert np.array_equal(out["0"], out["1"])


RES_TILE_CASES = [((64, 64, 17), (True, True, False), "const", 0), ((64, 64, 16), (True, True, True), "const", 0),
                  ((64, 64, 17), (True, True, False), "trans", 0), ((96, 64, 8), (True, True, True), "trans", 0),
                  ((128, 128, 17), (True, True, False), "const", 1), ((128, 128, 16), (True, True, True), "trans", 1)]


@pytest.mark.parametrize("dims,per,kind,level", RES_TILE_CASES)
def test_tiled_residual_is_the_colour_residual(dims, per, kind, level, monkeypatch):
    """The tiled residual (a CTA per plane tile, neighbours from shared
    memory) gives bit-for-bit the residual of the colour-interleaved kernel,
    and the same |res|^2 up to summation order: FP64 level residuals of the
    elastic and of a full non-symmetric shared stencil and of their
    plane-invariant coarse operators, Dirichlet and periodic z."""
    import stzpp_gb300 as sg
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per)
    st, fix = sg.elastic_stencil(1.0, 2.0, dx, dy, dz) if kind == "const" else trans_stencil(2, dx)
    out = {}
    for tile in ("0", "1"):   # 1: the tiled residual also in FP64
        monkeypatch.setenv("STZ_MG_TILE", tile)
        with sg.Multigrid(dims, per, precision="fp64", bottom="gs", max_coarse=5000) as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            N = mg.level_npts(level)
            rng = np.random.default_rng(9)
            mg.level_set_field(level, "x", rng.standard_normal((N, 3)))
            mg.level_set_field(level, "r", rng.standard_normal((N, 3)))
            out[tile] = mg.residual(level)
    assert np.array_equal(out["0"][0], out["1"][0])
    assert abs(out["0"][1] - out["1"][1]) <= 1e-12 * out["0"][1]


@pytest.mark.parametrize("dims,per,kind", [((128, 128, 33), (True, True, False), "const"),
                                             ((128, 128, 33), (True, True, False), "trans")])
def test_tiled_sweep_mixed_solve_bitwise(dims, per, kind, monkeypatch):
    """The FP32 V-cycles of the mixed solve with and without the tiled kernels
    (the tiled sweep and the tiled FP32 residual) give the same cycle count
    and the same solution bit for bit: the elastic and a full non-symmetric
    shared stencil, Dirichlet and periodic z."""
    import stzpp_gb300 as sg
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per, h=1.0 / m)   # isotropic: the cycle converges
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    out = {}
    for tile in ("0", "1"):   # 1: the tiled kernels on every level they apply to
        monkeypatch.setenv("STZ_MG_TILE", tile)
        with sg.Multigrid(dims, per, precision="mixed", sweep_growth=False) as mg:
            if kind == "const":
                mg.setup_matrices(*sg.elastic_stencil(1.0, 2.0, *h))
            else:
                mg.setup_matrices(*trans_stencil(2, h[0]))
            mg.setup_fields(r=b)
            cyc, rel = mg.solve(1e-10, 6, check=False)
            out[tile] = (cyc, rel, mg.get_x())
    assert np.isfinite(out["0"][1]) and out["0"][1] < 1e-3
    assert out["0"][:2] == out["1"][:2]
    assert np.array_equal(out["0"][2], out["1"][2])


BAND_LEVEL_CASES = [((64, 64, 17), (True, True, False), "const", 0, 2), ((64, 64, 16), (True, True, True), "const", 0, 2),
                    ((128, 64, 9), (True, True, False), "const", 0, 3), ((128, 128, 8), (True, True, True), "const", 0, 2),
                    ((256, 256, 9), (True, True, False), "const", 0, 2), ((64, 32, 5), (True, True, False), "const", 0, 4),
                    ((128, 128, 17), (True, True, False), "const", 1, 2), ((128, 128, 16), (True, True, True), "const", 1, 3),
                    ((128, 64, 17), (True, True, False), "trans", 1, 2), ((256, 128, 10), (True, True, False), "trans", 1, 2),
                    ((32, 32, 17), (True, True, False), "const", 0, 2), ((16, 16, 9), (True, True, False), "const", 0, 3),
                    ((64, 64, 33), (True, True, False), "const", 1, 2), ((64, 64, 16), (True, True, True), "trans", 1, 2),
                    ((128, 32, 9), (True, True, False), "const", 0, 3), ((256, 64, 16), (True, True, True), "trans", 1, 2)]


@pytest.mark.parametrize("dims,per,kind,level,sweeps", BAND_LEVEL_CASES)
def test_band_sweep_is_the_colour_sweep(dims, per, kind, level, sweeps, monkeypatch):
    """The band sweep (full-width bands of 8 rows, planes staged by TMA boxes,
    split at the periodic wrap in y) gives bit for bit the result of the eight
    colour launches: FP64 level sweeps of the elasticity stencil on the fine
    level and of the plane-invariant coarse operators (sparse elastic and
    full from a non-symmetric stencil) on level 1, Dirichlet and periodic z,
    8 to 128 sub-grid columns, two bands (both at the wrap) and many, even
    and odd sweep counts."""
    import stzpp_gb300 as sg
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    st, fix = sg.elastic_stencil(1.0, 2.0, *h) if kind == "const" else trans_stencil(2, h[0])
    out = {}
    for band in ("0", "1"):
        monkeypatch.setenv("STZ_MG_BAND", band)
        monkeypatch.setenv("STZ_MG_TILE", "0")
        with sg.Multigrid(dims, per, precision="fp64", bottom="gs", max_coarse=10 ** 6 if level == 0 else 5000) as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            assert (mg.sweep_kind(level)[0] == "band") == (band == "1")
            N = mg.level_npts(level)
            rng = np.random.default_rng(11)
            mg.level_set_field(level, "x", rng.standard_normal((N, 3)))
            mg.level_set_field(level, "r", rng.standard_normal((N, 3)))
            mg.gauss_seidel(level, sweeps)
            out[band] = mg.level_get_field(level, "x")
    assert np.array_equal(out["0"], out["1"])


@pytest.mark.parametrize("dims,per", [((128, 128, 33), (True, True, False)), ((256, 256, 17), (True, True, False)),
                                      ((128, 64, 24), (True, True, False))])
def test_band_sweep_mixed_solve_bitwise(dims, per, monkeypatch):
    """The FP32 V-cycles of the mixed solve with the band sweep on the fine
    level (the default) and with the colour launches give the same cycle
    count and the same solution bit for bit (an even plane count puts the
    upper plate on an odd plane)."""
    import stzpp_gb300 as sg
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per, h=1.0 / m)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    out = {}
    for band in ("0", "1"):
        monkeypatch.setenv("STZ_MG_BAND", band)
        with sg.Multigrid(dims, per, precision="mixed", sweep_growth=False, v_down=2, v_up=3) as mg:
            mg.setup_matrices(*sg.elastic_stencil(1.0, 2.0, *h))
            mg.setup_fields(r=b)
            cyc, rel = mg.solve(1e-10, 8, check=False)
            out[band] = (cyc, rel, mg.get_x())
    assert np.isfinite(out["0"][1]) and out["0"][1] < 1e-3
    assert out["0"][:2] == out["1"][:2]
    assert np.array_equal(out["0"][2], out["1"][2])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_cluster_tail_is_the_level_graph(precision, monkeypatch):
    """The persistent cluster kernels for the small levels (STZ_MG_TAIL=1:
    the down and up halves of the cycle below 300,000 nodes each in one
    thread-block cluster launch, cluster barriers between phases) give the
    per-level launches' cycle count and solution bit for bit."""
    import stzpp_gb300 as sg
    dims, per = (128, 128, 129), (True, True, False)
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    out = {}
    for tail in ("0", "1"):
        if tail == "1":
            monkeypatch.setenv("STZ_MG_TAIL", "1")
        else:
            monkeypatch.delenv("STZ_MG_TAIL", raising=False)
        with sg.Multigrid(dims, per, precision=precision, sweep_growth=False, v_down=2, v_up=3) as mg:
            mg.setup_matrices(*sg.elastic_stencil(1.0, 2.0, *h))
            mg.setup_fields(r=b)
            cyc, rel = mg.solve(1e-10, 30)
            out[tail] = (cyc, rel, mg.get_x())
    assert out["0"][:2] == out["1"][:2]
    assert np.array_equal(out["0"][2], out["1"][2])


@pytest.mark.parametrize("dims,kind,precision", [((64, 64, 65), "const", "fp64"), ((64, 64, 65), "trans", "fp64"),
                                                 ((32, 32, 33), "const", "mixed"), ((96, 64, 16), "trans", "fp64")])
def test_fourier_bottom_inverse_is_the_dense_inverse(dims, kind, precision, monkeypatch):
    """The bottom inverse of a plane-invariant operator periodic in x and y
    from its Fourier blocks (m n complex systems of order 3o) against the
    dense Gauss-Jordan inverse: the same cycle count, solutions to 1e-12,
    and the bottom level's operator applied to the inverse's output gives
    back its input (through whole solves: the reference's own hierarchy)."""
    import stzpp_gb300 as sg
    m, n, o = dims
    per = (True, True, False)
    h = P.grid_spacing(m, n, o, per, h=1.0 / m)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    st, fix = sg.elastic_stencil(1.0, 2.0, *h) if kind == "const" else trans_stencil(1, h[0])
    out = {}
    for fourier in ("0", "1"):
        monkeypatch.setenv("STZ_MG_BOTTOM_FOURIER", fourier)
        with sg.Multigrid(dims, per, precision=precision, sweep_growth=False, v_down=2, v_up=3) as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            mg.setup_fields(r=b)
            cyc, rel = mg.solve(1e-12 if precision == "fp64" else 1e-10, 60)
            out[fourier] = (cyc, mg.get_x())
    assert out["0"][0] == out["1"][0]
    x0, x1 = out["0"][1], out["1"][1]
    assert np.linalg.norm(x1 - x0) <= 1e-11 * np.linalg.norm(x0)


@pytest.mark.parametrize("bandres", ["default", "1"])
@pytest.mark.parametrize("dims,per,kind", [((128, 128, 33), (True, True, False), "const"),
                                          ((128, 64, 24), (True, True, False), "trans"),
                                          ((64, 64, 32), (True, True, False), "const")])
def test_band_kernels_fp64_solve_bitwise(dims, per, kind, bandres, monkeypatch):
    """FP64 solves with the band kernels forced (STZ_MG_BAND=1: the band sweep
    on every level it serves and the band residual on the plane-invariant
    ones, or with STZ_MG_BAND_RES=1 on the fine level too) and without: the
    same cycle count and the same solution bit for bit."""
    import stzpp_gb300 as sg
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per, h=1.0 / m)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    st, fix = sg.elastic_stencil(1.0, 2.0, *h) if kind == "const" else trans_stencil(1, h[0])
    if bandres != "default":
        monkeypatch.setenv("STZ_MG_BAND_RES", bandres)
    out = {}
    for band in ("0", "1"):
        monkeypatch.setenv("STZ_MG_BAND", band)
        with sg.Multigrid(dims, per, precision="fp64", sweep_growth=False, v_down=2, v_up=2) as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            mg.setup_fields(r=b)
            cyc, rel = mg.solve(1e-10, 6, check=False)
            out[band] = (cyc, rel, mg.get_x())
    assert out["0"][:2] == out["1"][:2]
    assert np.array_equal(out["0"][2], out["1"][2])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("dims,per,kind", [((128, 128, 33), (True, True, False), "const"),
                                          ((128, 64, 32), (True, True, False), "const"),
                                          ((64, 64, 16), (True, True, True), "const"),
                                          ((128, 64, 25), (True, True, False), "trans"),
                                          ((256, 256, 17), (True, True, False), "const")])
def test_fused_residual_restriction_is_the_two_kernels(dims, per, kind, precision, monkeypatch):
    """The descent's residual and restriction in one pass (opt-in with
    STZ_MG_FUSED_RESTRICT=1; the residual never written) against the
    residual kernel followed by the restriction kernel:
    the same iterate bit for bit after three V-cycles -- FP32 V-cycles of the
    mixed solver and FP64 ones (STZ_MG_TILE=1, the tiled kernels in FP64
    too), the elastic and a full non-symmetric shared stencil, an odd and an
    even Dirichlet z (the even one puts the last fine plane under the last
    coarse plane alone) and a periodic z (singular with x and y periodic:
    GS at the bottom, no solve to a tolerance)."""
    import stzpp_gb300 as sg
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per, h=1.0 / m)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    st, fix = sg.elastic_stencil(1.0, 2.0, *h) if kind == "const" else trans_stencil(1, h[0])
    if precision == "fp64":
        monkeypatch.setenv("STZ_MG_TILE", "1")
    out = {}
    for fused in ("0", "1"):
        monkeypatch.setenv("STZ_MG_FUSED_RESTRICT", fused)
        with sg.Multigrid(dims, per, precision=precision, sweep_growth=False, v_down=2, v_up=2, bottom="gs") as mg:
            mg.setup_matrices(stencil=st, fix=fix)
            mg.setup_fields(r=b)
            for _ in range(3):
                mg.v_cycle()
            out[fused] = mg.get_x()
    assert np.all(np.isfinite(out["0"])) and np.linalg.norm(out["0"]) > 0
    assert np.array_equal(out["0"], out["1"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hierarchy_stops_before_an_odd_periodic_level(precision, oracle_port):
    """72x72x17, periodic x and y: the halving chain 72 -> 36 -> 18 -> 9 would
    reach an odd periodic size above max_coarse (18x18x5 = 1620 nodes), which
    the 8-colour smoother cannot take; the hierarchy stops at 18x18x5, and
    the converged solution matches the reference's lexicographic solver with
    its own hierarchy (which goes on to 9x9x3)."""
    import stzpp_gb300 as sg
    dims, per = (72, 72, 17), (True, True, False)
    m, n, o = dims
    dx, dy, dz = P.grid_spacing(m, n, o, per, h=1.0 / m)   # isotropic: the cycles converge
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, dx, dy, dz)
    st, fix = P.elastic_stencil_const(1.0, 2.0, dx, dy, dz)
    ref = oracle_port.PortMultigrid(dims, per, stencil=st, fix=fix, max_coarse=1024)
    ref.set_field(0, "r", b)
    ref.set_field(0, "x", np.zeros_like(b))
    cyc_ref, hist = ref.solve(1e-13, 100, bottom="gs", smoother="lex")
    assert hist[cyc_ref - 1] <= 1e-13
    x_ref = ref.get_field(0, "x")
    with sg.Multigrid(dims, per, precision=precision) as mg:
        assert mg.nlevels == 3
        assert mg.level_npts(2) == 18 * 18 * 5
        mg.setup_matrices(*sg.elastic_stencil(1.0, 2.0, dx, dy, dz))
        mg.setup_fields(r=b)
        cycles, rel = mg.solve(1e-10, 100)
        x = mg.get_x()
    assert rel <= 1e-10
    err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    assert err <= SOLUTION_RTOL, f"{precision}: {cycles} cycles, error {err:.3e}"
