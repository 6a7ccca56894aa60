"""Generates the golden fixtures of the multigrid from the compiled reference.

Needs oracle/_ref/libstzref.so, i.e. the reference's own mg_3d_template
sources compiled by ``make -C oracle ref`` where the reference checkout is
available.  Writes tests/golden/reference_small.npz, which the CPU tests use
to pin the C restatement of the reference (oracle/stzmg_oracle.c) on machines
without the reference.

Cases (all seeded):
  * ``p110``: 8x8x9, periodic x,y, Dirichlet z, constant elasticity stencil
    (mu=1, lambda=2, dx=1/8), hierarchy extended to 2x2x3 (max_coarse 16);
  * ``d000``: 6x5x4, all Dirichlet (even sizes: the collapse masks and the
    restrict_partial mask-145 quirk), hierarchy to <= 8 nodes;
  * ``var``: 8x8x9 periodic x,y with lognormal mu (seed 1), lambda = 2 mu,
    per-node stencils through fill_entries;
  * ``cfg1``: the 32x32x33 problem (dx=1/32), reference hierarchy and cycle
    (lexicographic GS, 24 bottom sweeps): residual history of the solve to
    1e-10 and a strided subsample of the solution.
For each small case: box bounds S and coefficients of every level, one GS
sweep, restriction, interpolation and two V-cycles from seeded fields.

Also ``trans``: the reference's transformed-frame stencils of trans_sim_3d
for a few frames (the coefficient-change path), from its generated
stenc_funcs.hh -> tests/golden/trans_stencils.npz.

Also ``adv``: the reference's quasi-static advection step
(shear_sim_3d::advection_step) run once through oracle/_ref/libstzadv.so
(``make -C oracle advref``) on seeded ghosted grids -> tests/golden/adv_step.npz
(inputs and the changed Field members of every point).

Also ``out``: the files the reference's own writers produce -- every
Field member of shear_sim_3d::output_cube on a seeded 6x5x4 grid, and the
x, r and residual z-slices of region::output_internal on an 8x6x5 multigrid
level -> tests/golden/output_files.npz (inputs and file bytes).

Also ``proj``: the reference's r_field and its whole quasi-static projection
step (shear_sim_3d::projection_step: multigrid solve, stress update,
proj_mag) through oracle/_ref/libstzadv.so -> tests/golden/proj_step.npz.

Run: python tests/golden/make_golden.py [trans | adv | out | proj]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import problem as P  # noqa: E402
from oracle import refpy  # noqa: E402


def build(dims, per, kind, max_coarse):
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    if kind == "const":
        st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
        return refpy.RefMultigrid(dims, per, stencil=st, fix=fix, max_coarse=max_coarse)
    mu = P.lognormal_mu(1, m, n, o)
    return refpy.RefMultigrid(dims, per, points=P.elastic_stencil_points(mu, 2 * mu, *h, per), max_coarse=max_coarse)


def small_case(out, name, dims, per, kind, max_coarse):
    R = build(dims, per, kind, max_coarse)
    L = R.nlevels
    out[f"{name}/nlevels"] = np.int32(L)
    for l in range(L):
        out[f"{name}/dims{l}"] = np.array(R.level_dims(l), dtype=np.int32)
        out[f"{name}/S{l}"] = R.level_S(l).astype(np.int8)
        if l > 0:
            out[f"{name}/A{l}"] = R.level_A(l)
    rng = np.random.default_rng(11)
    N0 = R.npts(0)
    x0, b0 = rng.standard_normal((N0, 3)), rng.standard_normal((N0, 3))
    out[f"{name}/x0"], out[f"{name}/b0"] = x0, b0
    R.set_field(0, "x", x0)
    R.set_field(0, "r", b0)
    R.gauss_seidel(0, 1)
    out[f"{name}/gs0"] = R.get_field(0, "x")
    R.restriction(1)
    out[f"{name}/restrict1"] = R.get_field(1, "r")
    xc = rng.standard_normal((R.npts(1), 3))
    out[f"{name}/xc1"] = xc
    R.set_field(1, "x", xc)
    R.interpolation(1)
    out[f"{name}/interp0"] = R.get_field(0, "x")
    R.set_field(0, "x", x0)
    R.set_field(0, "r", b0)
    R.v_cycle("gs")
    R.v_cycle("gs")
    out[f"{name}/vcycle2"] = R.get_field(0, "x")
    R.close()


# transforms of the trans_sim frame for the coefficient-change fixtures
TRANS_T = [[[1.0, 0.0, 0.3], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
           [[1.0, 0.0, 0.1], [0.0, 1.0, -0.2], [0.0, 0.0, 1.0]],
           [[1.05, 0.02, 0.15], [0.0, 0.97, 0.05], [0.0, 0.0, 1.0]]]


def trans_stencils(path):
    """Stencils of trans_sim_3d::set_up_stencil_and_matrices for the TRANS_T
    frames (mu = 1, lambda = 2, dt = 1, dx = dy = dz = 1), computed by the
    reference's generated functions (oracle/trans_stencil.py builds them)."""
    import ctypes
    lib_path = os.path.join(ROOT, "oracle", "_ref", "libtransstencil.so")
    if not os.path.exists(lib_path):
        sys.exit("oracle/_ref/libtransstencil.so is missing: run `python oracle/trans_stencil.py <reference>/src`")
    lib = ctypes.CDLL(lib_path)
    lib.ref_trans_stencil.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 6 + [ctypes.c_void_p] * 2
    T = np.array(TRANS_T)
    S = np.zeros((len(T), 243))
    F = np.zeros((len(T), 9))
    for c in range(len(T)):
        t = np.ascontiguousarray(T[c])
        lib.ref_trans_stencil(t.ctypes.data_as(ctypes.c_void_p), 1.0, 2.0, 1.0, 1.0, 1.0, 1.0,
                              S[c].ctypes.data_as(ctypes.c_void_p), F[c].ctypes.data_as(ctypes.c_void_p))
    np.savez_compressed(path, T=T, stencil=S, fix=F)
    print("wrote", path)


# (name, interior dims, seed, dt, stress bias toward yield)
ADV_CASES = [("elastic", (6, 5, 4), 3, 500.0, -0.5), ("mixed", (7, 6, 5), 0, 500.0, 0.0),
             ("plastic", (6, 6, 4), 2, 50.0, 1.2), ("long", (5, 4, 6), 1, 2000.0, 0.6)]
ADV_IN = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 19, 27]        # u v w s11..s33 chi cchi ad_Dpl
ADV_OUT = [13, 14, 15, 16, 17, 18, 19, 26, 27]          # cs11..cs33 cchi sbar ad_Dpl


def adv_steps(path):
    from oracle import advect as A
    if not A.reference_available():
        sys.exit("oracle/_ref/libstzadv.so is missing: run `make -C oracle advref` where the reference is available")
    out = {}
    for name, (nx, ny, nz), seed, dt, bias in ADV_CASES:
        prm = A.driver_params(nx)
        F = A.random_fields(seed, nx, ny, nz, sigma_scale=0.7 if bias >= 0 else 0.2, plastic_bias=max(bias, 0.0))
        R = A.reference_step(F, nx, ny, nz, prm, dt)
        out[name + "/dims"] = np.array([nx, ny, nz])
        out[name + "/dt"] = np.float64(dt)
        out[name + "/params"] = np.array([prm[k] for k in A.PARAM_NAMES])
        out[name + "/in"] = F[:, ADV_IN]
        out[name + "/out"] = R[:, ADV_OUT]
        print(name, "cells above the yield stress:", int((A.interior(R, nx, ny, nz)[..., 27] > 0).sum()),
              "of", nx * ny * nz)
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


# (name, cells nx ny nz, seed, dt, stress scale): quasi-static projection steps
PROJ_CASES = [("a", (8, 6, 5), 4, 0.002, 0.5), ("b", (12, 10, 8), 7, 0.01, 0.2)]


def projection_steps(path):
    """The reference's r_field of every node and its whole projection step
    (multigrid solve, stress update, proj_mag) on seeded ghosted grids, x and
    y periodic with z plates: inputs (cell stresses), and outputs (node
    right-hand side, solved node velocities, new cell stresses, proj_mag)."""
    from oracle import advect as A
    if not A.reference_available():
        sys.exit("oracle/_ref/libstzadv.so is missing: run `make -C oracle advref` where the reference is available")
    out = {}
    for name, (nx, ny, nz), seed, dt, scale in PROJ_CASES:
        prm = A.driver_params(nx)
        F = A.random_fields(seed, nx, ny, nz, sigma_scale=scale)
        r = A.reference_rhs(F, nx, ny, nz, prm)
        G, pm = A.reference_projection(F, nx, ny, nz, prm, dt)
        out[name + "/cells"] = np.array([nx, ny, nz])
        out[name + "/dt"] = np.float64(dt)
        out[name + "/lamb_mu"] = np.array([prm["lamb"], prm["mu"]])
        out[name + "/sigma"] = A.cell_stresses(F, nx, ny, nz)
        out[name + "/rhs"] = r
        out[name + "/u"] = A.node_velocities(G, nx, ny, nz)
        out[name + "/sigma_new"] = A.cell_stresses(G, nx, ny, nz)
        out[name + "/proj_mag"] = np.float64(pm)
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


OUT_CUBE = (6, 5, 4)
OUT_SLICE = ((8, 6, 5), (True, True, False), 2, [(0.0, 7.0, 0.0, 5.0), (0.0, 1.0, -0.5, 0.5)])
OUT_COLS = list(range(10)) + [20, 21, 22]   # u v w s11..s33 chi xi_x xi_y xi_z


def output_files(path):
    import tempfile
    from oracle import advect as A
    if not (A.reference_available() and refpy.available()):
        sys.exit("oracle/_ref/libstzadv.so and libstzref.so are needed: `make -C oracle ref advref`")
    out = {}
    d = tempfile.mkdtemp()
    nx, ny, nz = OUT_CUBE
    F = A.random_fields(21, nx, ny, nz, plastic_bias=0.5)
    F[:, 20:23] = np.random.default_rng(22).normal(size=(F.shape[0], 3))
    out["cube/in"] = F[:, OUT_COLS]
    for mode in range(16):
        A.reference_cube(F, nx, ny, nz, A.driver_params(nx), mode, os.path.join(d, "cube"), f"m{mode}", 3)
        out[f"cube/{mode}"] = np.frombuffer(open(os.path.join(d, "cube", f"m{mode}_grid.3"), "rb").read(), np.uint8)
    dims, per, k, boxes = OUT_SLICE
    st, fix = P.elastic_stencil_const(1.0, 2.0, 1 / dims[0], 1 / dims[1], 1 / (dims[2] - 1))
    R = refpy.RefMultigrid(dims, per, stencil=st, fix=fix, max_coarse=16)
    rng = np.random.default_rng(23)
    x, r = rng.normal(size=(int(np.prod(dims)), 3)), rng.normal(size=(int(np.prod(dims)), 3))
    R.set_field(0, "x", x)
    R.set_field(0, "r", r)
    out["slice/x"], out["slice/r"] = x, r
    for which in ("x", "r", "residual"):
        for b, box in enumerate(boxes):
            fn = os.path.join(d, f"{which}{b}")
            R.residual(0)   # the periodic ghosts output_residual reads
            R.output_slice(which, k, box, fn)
            out[f"slice/{which}/{b}"] = np.frombuffer(open(fn, "rb").read(), np.uint8)
    R.close()
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "out":
        output_files(os.path.join(HERE, "output_files.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "proj":
        projection_steps(os.path.join(HERE, "proj_step.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "adv":
        adv_steps(os.path.join(HERE, "adv_step.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "trans":
        trans_stencils(os.path.join(HERE, "trans_stencils.npz"))
        return
    if not refpy.available():
        sys.exit("oracle/_ref/libstzref.so is missing: run `make -C oracle ref` where the reference is available")
    out = {}
    small_case(out, "p110", (8, 8, 9), (True, True, False), "const", 16)
    small_case(out, "d000", (6, 5, 4), (False, False, False), "const", 8)
    small_case(out, "var", (8, 8, 9), (True, True, False), "var", 16)
    # the 32x32x33 problem with the reference's own solver
    m, n, o = 32, 32, 33
    per = (True, True, False)
    h = P.grid_spacing(m, n, o, per)
    b = P.rhs_divergence(P.random_strain(0, m, n, o, per), m, n, o, per, *h)
    R = build((m, n, o), per, "const", 1024)
    R.set_field(0, "r", b)
    R.set_field(0, "x", np.zeros_like(b))
    cycles, hist = R.solve(1e-10, 100)
    x = R.get_field(0, "x")
    out["cfg1/hist"] = hist
    out["cfg1/x_sub"] = x[::97]
    out["cfg1/x_norm"] = np.float64(np.linalg.norm(x))
    out["cfg1/b_norm"] = np.float64(np.linalg.norm(b))
    R.close()
    path = os.path.join(HERE, "reference_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes;", "cfg1 cycles", cycles)


if __name__ == "__main__":
    main()
