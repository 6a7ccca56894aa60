"""The quasi-static advection step of shear_sim_3d on the CPU, for tests.

Test infrastructure only.  Two implementations of shear_sim_3d::advection_step
(src/shear_sim_3d.cpp:393-525) on the reference's ghosted grid of Field points
(28 doubles per point, src/field.hh:10-23, 2 ghost layers, x fastest):

* :func:`port_step` -- the C restatement oracle/stzadv_oracle.c (in
  oracle/liboracle.so, built everywhere);
* :func:`reference_step` -- the unmodified reference step through
  oracle/adv_harness.cc (oracle/_ref/libstzadv.so, built only where the
  reference checkout exists).

Also the problem data the tests use: the reference driver's nondimensional
STZ parameters (src/shear_sim.cpp:31-81) and seeded random fields whose
ghost layers are periodic in x and y.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(_HERE, "_ref", "libstzadv.so")
NGHOST = 2
NFIELD = 28
# Field members (field.hh:11-22)
U, V, W, S11, S12, S13, S22, S23, S33, CHI = range(10)
CS11, CS12, CS13, CS22, CS23, CS33, CCHI = 13, 14, 15, 16, 17, 18, 19
SBAR, ADPL = 26, 27
STRESS = [S11, S12, S13, S22, S23, S33]
DSTRESS = [CS11, CS12, CS13, CS22, CS23, CS33]
PARAM_NAMES = ("mu", "sy", "tau0", "eps0", "c0", "delta", "omega", "bath_temp", "chi_inf", "ez", "diff_l")


class AdvPar(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double)] + \
               [(n, ctypes.c_double) for n in PARAM_NAMES]


def driver_params(nx, lx=1.0):
    """The STZ parameters of the reference driver in its units (stresses in
    units of the yield stress, times in units of the shear-wave time;
    shear_sim.cpp:31-81), with the diffusion length of 1.5 cells there."""
    TZ, kb = 21000.0, 1.3806503e-23
    sy_dim, E, nu, rho_dim = 0.85e9, 101e9, 0.35, 6125.0
    mu_dim = E / (2 * (1 + nu))
    ts = 1e-2 / np.sqrt(mu_dim / rho_dim)
    K = E / (3 * (1 - 2 * nu)) / sy_dim
    mu = mu_dim / sy_dim
    return {"mu": mu, "lamb": K - (2. / 3.) * mu, "sy": 1.0, "tau0": 1e-13 / ts, "c0": .4, "eps0": .3,
            "delta": 8000 / TZ, "omega": 300 * 26. / 17. * 1e-30 * sy_dim / (TZ * kb), "bath_temp": 400 / TZ,
            "chi_inf": 900 / TZ, "ez": 1.0, "diff_l": 1.5 * lx / nx}


def random_fields(seed, nx, ny, nz, sigma_scale=0.7, vel_scale=1e-3, plastic_bias=0.0):
    """Seeded Field array of the ghosted grid (npoints, 28): node velocities,
    cell stresses (a fraction above the yield stress), chi around 550 K,
    previous ad_Dpl; ghost layers periodic in x and y, random in z."""
    g = NGHOST
    rng = np.random.default_rng(seed)
    F = np.zeros((nz + 2 * g, ny + 2 * g, nx + 2 * g, NFIELD))
    core = F[g:g + nz, g:g + ny, g:g + nx]
    core[..., U:W + 1] = rng.normal(0, vel_scale, core[..., U:W + 1].shape)
    core[..., S11:S33 + 1] = rng.normal(0, sigma_scale, core[..., S11:S33 + 1].shape)
    core[..., S11:S33 + 1] += plastic_bias * np.array([0, 1, 0, 0, 0, 0])
    core[..., CHI] = 550 / 21000 + rng.normal(0, 15 / 21000, core[..., CHI].shape)
    core[..., ADPL] = rng.uniform(0, 1e-3, core[..., ADPL].shape)
    # x and y ghosts: periodic copies; z ghosts: random values of the same kind
    F[g:g + nz, g:g + ny, :g] = F[g:g + nz, g:g + ny, nx:nx + g]
    F[g:g + nz, g:g + ny, nx + g:] = F[g:g + nz, g:g + ny, g:2 * g]
    F[g:g + nz, :g] = F[g:g + nz, ny:ny + g]
    F[g:g + nz, ny + g:] = F[g:g + nz, g:2 * g]
    for zs in (slice(0, g), slice(nz + g, nz + 2 * g)):
        shp = F[zs].shape[:-1]
        F[zs, ..., U:W + 1] = rng.normal(0, vel_scale, shp + (3,))
        F[zs, ..., S11:S33 + 1] = rng.normal(0, sigma_scale, shp + (6,))
        F[zs, ..., CHI] = 550 / 21000 + rng.normal(0, 15 / 21000, shp)
        F[zs, ..., ADPL] = rng.uniform(0, 1e-3, shp)
    return F.reshape(-1, NFIELD)


def interior(F, nx, ny, nz):
    """The interior points of a ghosted (npoints, ...) array, as (nz, ny, nx, ...)."""
    g = NGHOST
    A = F.reshape((nz + 2 * g, ny + 2 * g, nx + 2 * g) + F.shape[1:])
    return A[g:g + nz, g:g + ny, g:g + nx]


def _par(nx, ny, nz, lx, ly, lz, prm):
    return AdvPar(nx, ny, nz, lx / nx, ly / ny, lz / nz, *[prm[n] for n in PARAM_NAMES])


def port_step(fields, nx, ny, nz, prm, dt, lx=1.0, ly=1.0, lz=1.0):
    """One step of the C restatement on a copy of fields; (new fields, yielded)."""
    from oracle import port
    lib = port._load()
    lib.so_adv_step.argtypes = [ctypes.c_void_p, ctypes.POINTER(AdvPar), ctypes.c_double]
    out = np.ascontiguousarray(fields, dtype=np.float64).copy()
    par = _par(nx, ny, nz, lx, ly, lz, prm)
    y = lib.so_adv_step(out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(par), dt)
    return out, bool(y)


def reference_available() -> bool:
    return os.path.exists(REF_LIB)


def _ref_lib():
    lib = ctypes.CDLL(REF_LIB)
    vp = ctypes.c_void_p
    lib.adv_new.restype = vp
    lib.adv_new.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [vp, ctypes.c_int, ctypes.c_char_p]
    lib.adv_output_cube.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    return lib


def _ref_params(prm):
    return np.array([prm["mu"], prm["lamb"], prm["sy"], prm["tau0"], prm["c0"], prm["eps0"], prm["delta"],
                     prm["omega"], prm["bath_temp"], prm["chi_inf"], prm["ez"], prm["diff_l"]])


def reference_cube(fields, nx, ny, nz, prm, mode, outdir, prefix, frame):
    """The unmodified reference's output_cube of Field member `mode` for the
    Field array `fields`, appended to <outdir>/<prefix>_grid.<frame>."""
    lib = _ref_lib()
    vp = ctypes.c_void_p
    p = _ref_params(prm)
    h = lib.adv_new(nx, ny, nz, 1.0, 1.0, 1.0, p.ctypes.data_as(vp), 0, outdir.encode())
    try:
        buf = np.ascontiguousarray(fields, dtype=np.float64).copy()
        lib.adv_set(h, buf.ctypes.data_as(vp))
        lib.adv_output_cube(h, prefix.encode(), mode, frame)
    finally:
        lib.adv_free(h)


def cube_values(fields, nx, ny, nz, mode):
    """numpy restatement of output_cube's values (Field::fval, field.hh:157-177;
    x slowest, z fastest; node-based members include the top z node), float32."""
    g = NGHOST
    zsize = nz + 1 if (mode <= 2 or mode >= 13) else nz
    A = fields.reshape(nz + 2 * g, ny + 2 * g, nx + 2 * g, NFIELD)[g:g + zsize, g:g + ny, g:g + nx]
    if mode in (9, 10):
        s11, s22, s33 = A[..., S11], A[..., S22], A[..., S33]
        p = -((s11 + s22) + s33) * (1 / 3.)
        if mode == 9:
            v = p
        else:
            t11, t22, t33 = s11 + p, s22 + p, s33 + p
            q = 0.5 * ((t11 * t11 + t22 * t22) + t33 * t33)
            q = ((q + A[..., S12] * A[..., S12]) + A[..., S13] * A[..., S13]) + A[..., S23] * A[..., S23]
            v = np.sqrt(q)
    elif mode == 12:
        v = A[..., CHI] * 21000.
    else:
        v = A[..., {11: CHI, 13: 20, 14: 21, 15: 22}.get(mode, mode)]
    return np.ascontiguousarray(v.transpose(2, 1, 0)).astype(np.float32).reshape(-1)


def reference_step(fields, nx, ny, nz, prm, dt, lx=1.0, ly=1.0, lz=1.0, zper=False):
    """One step of the unmodified reference on a copy of fields."""
    lib = _ref_lib()
    vp = ctypes.c_void_p
    lib.adv_npoints.argtypes = [vp]
    lib.adv_npoints.restype = ctypes.c_long
    lib.adv_set.argtypes = lib.adv_get.argtypes = [vp, vp]
    lib.adv_step.argtypes = [vp, ctypes.c_double]
    lib.adv_free.argtypes = [vp]
    p = _ref_params(prm)
    h = lib.adv_new(nx, ny, nz, lx, ly, lz, p.ctypes.data_as(vp), int(zper), b"adv_harness_out")
    try:
        assert lib.adv_npoints(h) == fields.shape[0]
        buf = np.ascontiguousarray(fields, dtype=np.float64).copy()
        lib.adv_set(h, buf.ctypes.data_as(vp))
        lib.adv_step(h, dt)
        lib.adv_get(h, buf.ctypes.data_as(vp))
    finally:
        lib.adv_free(h)
    return buf


def _ref_handle(lib, fields, nx, ny, nz, prm, zper=False, outdir="adv_harness_out"):
    vp = ctypes.c_void_p
    lib.adv_npoints.argtypes = [vp]
    lib.adv_npoints.restype = ctypes.c_long
    lib.adv_set.argtypes = lib.adv_get.argtypes = [vp, vp]
    lib.adv_free.argtypes = [vp]
    p = _ref_params(prm)
    h = lib.adv_new(nx, ny, nz, 1.0, 1.0, 1.0, p.ctypes.data_as(vp), int(zper), outdir.encode())
    assert lib.adv_npoints(h) == fields.shape[0]
    buf = np.ascontiguousarray(fields, dtype=np.float64).copy()
    lib.adv_set(h, buf.ctypes.data_as(vp))
    return h, buf


def reference_rhs(fields, nx, ny, nz, prm):
    """The unmodified reference's r_field (shear_sim_3d.hh:283-385) of every
    node of an nx x ny x nz cell grid (x, y periodic, z plates): (npts, 3),
    nodes in natural order with nz + 1 node planes."""
    lib = _ref_lib()
    vp = ctypes.c_void_p
    lib.adv_rhs.argtypes = [vp, vp]
    h, _ = _ref_handle(lib, fields, nx, ny, nz, prm)
    try:
        out = np.zeros((nx * ny * (nz + 1), 3))
        lib.adv_rhs(h, out.ctypes.data_as(vp))
    finally:
        lib.adv_free(h)
    return out


def reference_projection(fields, nx, ny, nz, prm, dt):
    """The unmodified reference's quasi-static projection step
    (shear_sim_3d::projection_step, shear_sim_3d.cpp:528-724: multigrid solve
    for the velocities, then the stress update) on a copy of fields;
    returns (new fields, proj_mag)."""
    lib = _ref_lib()
    vp = ctypes.c_void_p
    lib.adv_project.argtypes = [vp, ctypes.c_double]
    lib.adv_project.restype = ctypes.c_double
    import shutil
    import tempfile
    d = tempfile.mkdtemp()   # the step appends its proj_mag.dat there
    h, buf = _ref_handle(lib, fields, nx, ny, nz, prm, outdir=d)
    try:
        pm = lib.adv_project(h, dt)
        lib.adv_get(h, buf.ctypes.data_as(vp))
    finally:
        lib.adv_free(h)
        shutil.rmtree(d, ignore_errors=True)
    return buf, pm


def node_velocities(fields, nx, ny, nz):
    """(npts, 3) node velocities u, v, w of a ghosted Field array, nodes in
    natural order with nz + 1 node planes (the top plate included)."""
    g = NGHOST
    A = fields.reshape(nz + 2 * g, ny + 2 * g, nx + 2 * g, NFIELD)
    return np.ascontiguousarray(A[g:g + nz + 1, g:g + ny, g:g + nx, U:W + 1]).reshape(-1, 3)


def cell_stresses(fields, nx, ny, nz):
    """(nz, ny, nx, 6) cell stresses s11 s12 s13 s22 s23 s33 of a ghosted Field array."""
    return np.ascontiguousarray(interior(fields, nx, ny, nz)[..., S11:S33 + 1])
