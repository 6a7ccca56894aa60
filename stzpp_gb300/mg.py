"""Python mirror of the reference multigrid interface over the stz_mg C-ABI.

The reference's multigrid<vec3, M> (mg_3d_template/multigrid.hh) is driven by
the simulation as::

    multigrid<vec3,M> mgrid(sim, buf);   // hierarchy
    mgrid.setup_matrices(sim);           // operators + RAT
    mgrid.setup_fields(sim);             // x, r
    mgrid.v_cycle();                     // until reg[0]->l2_error_all() < tol
    ... reg[0]->x0 ...                   // solution

:class:`Multigrid` offers the same calls on the GPU, through ``libstz_mg.so``
(include/stz_mg.h).  Arrays are natural order (x fastest), 3 doubles per node.
Host arrays may be numpy arrays; device arrays may be CUDA torch tensors
(float64, contiguous), passed by pointer without a copy.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libstz_mg.so")

OK, ERR_ARG, ERR_CUDA, ERR_UNSUPPORTED, ERR_NOCONV, ERR_SINGULAR, ERR_NONFINITE, ERR_OOM = range(8)
FP64, MIXED = 0, 1
BOTTOM_DIRECT, BOTTOM_GS = 0, 1
HOST, DEVICE = 0, 1
FIELD_X, FIELD_R, FIELD_RES = 0, 1, 2
_FIELDS = {"x": FIELD_X, "r": FIELD_R, "res": FIELD_RES}

# every entry point declared in include/stz_mg.h
EXPORTS = (
    "stz_mg_desc_default", "stz_mg_last_error", "stz_mg_create", "stz_mg_destroy",
    "stz_mg_set_stencil_const", "stz_mg_set_stencil_points", "stz_mg_set_coeffs_lame", "stz_mg_setup",
    "stz_mg_set_rhs", "stz_mg_set_x", "stz_mg_get_x", "stz_mg_get_rhs", "stz_mg_set_rhs_divergence",
    "stz_mg_vcycle", "stz_mg_solve",
    "stz_mg_solve_stats", "stz_mg_residual_norm", "stz_mg_l2_error_all", "stz_mg_num_levels", "stz_mg_level_dims",
    "stz_mg_level_operator", "stz_mg_level_set_field", "stz_mg_level_get_field",
    "stz_mg_level_gauss_seidel", "stz_mg_level_restriction", "stz_mg_level_interpolation",
    "stz_mg_level_get_planes", "stz_mg_level_set_planes", "stz_mg_level_gs_colours", "stz_mg_level_restrict_residual",
    "stz_mg_level_residual", "stz_mg_time_kernel", "stz_mg_sweep_kind", "stz_mg_const_residual_sumsq_noalloc",
    "stz_mg_adjoint_solve", "stz_mg_coeff_grad", "stz_mg_stress_update", "stz_mg_advection_step",
    "stz_mg_output_slice", "stz_mg_cube_values", "stz_mg_output_cube",
)

# measurement hook kernel ids (include/stz_mg.h)
K_GS_COLOUR, K_RESIDUAL, K_RESTRICT, K_INTERP, K_RESIDUAL64, K_GS_SWEEP = range(6)


class StzMgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"stz_mg error {code}: {msg}")
        self.code = code


class Desc(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int), ("n", ctypes.c_int), ("o", ctypes.c_int),
                ("x_prd", ctypes.c_int), ("y_prd", ctypes.c_int), ("z_prd", ctypes.c_int),
                ("precision", ctypes.c_int), ("v_down", ctypes.c_int), ("v_up", ctypes.c_int),
                ("max_coarse", ctypes.c_int), ("bottom", ctypes.c_int), ("bottom_sweeps", ctypes.c_int),
                ("sweep_growth", ctypes.c_int), ("device", ctypes.c_int), ("stream", ctypes.c_void_p)]


_lib = None


def load_library():
    """Loads libstz_mg.so; raises if it has not been built (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m stzpp_gb300.build`")
    lib = ctypes.CDLL(LIB_PATH)
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.stz_mg_desc_default.argtypes = [ctypes.POINTER(Desc)]
    lib.stz_mg_desc_default.restype = None
    lib.stz_mg_last_error.restype = ctypes.c_char_p
    lib.stz_mg_create.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(vp)]
    lib.stz_mg_destroy.argtypes = [vp]
    lib.stz_mg_set_stencil_const.argtypes = [vp, vp, vp]
    lib.stz_mg_set_stencil_points.argtypes = [vp, vp, ci]
    lib.stz_mg_set_coeffs_lame.argtypes = [vp, vp, vp, cd, cd, cd, cd, ci]
    lib.stz_mg_setup.argtypes = [vp]
    lib.stz_mg_set_rhs_divergence.argtypes = [vp, vp, cd, cd, cd, ci]
    for f in ("stz_mg_set_rhs", "stz_mg_set_x", "stz_mg_get_x", "stz_mg_get_rhs"):
        getattr(lib, f).argtypes = [vp, vp, ci]
    lib.stz_mg_vcycle.argtypes = [vp]
    lib.stz_mg_solve.argtypes = [vp, cd, ci, ctypes.POINTER(ci), ctypes.POINTER(cd)]
    lib.stz_mg_solve_stats.argtypes = [vp, ctypes.POINTER(ci), ctypes.POINTER(ci), ctypes.POINTER(ctypes.c_longlong)]
    lib.stz_mg_residual_norm.argtypes = [vp, ctypes.POINTER(cd), ctypes.POINTER(cd)]
    lib.stz_mg_l2_error_all.argtypes = [vp, ctypes.POINTER(cd)]
    lib.stz_mg_num_levels.argtypes = [vp, ctypes.POINTER(ci)]
    lib.stz_mg_level_dims.argtypes = [vp, ci, vp]
    lib.stz_mg_level_operator.argtypes = [vp, ci, vp, vp]
    lib.stz_mg_level_set_field.argtypes = [vp, ci, ci, vp, ci]
    lib.stz_mg_level_get_field.argtypes = [vp, ci, ci, vp, ci]
    lib.stz_mg_level_gauss_seidel.argtypes = [vp, ci, ci]
    lib.stz_mg_level_restriction.argtypes = [vp, ci]
    lib.stz_mg_level_get_planes.argtypes = [vp, ci, ci, ci, ci, vp, ci]
    lib.stz_mg_level_set_planes.argtypes = [vp, ci, ci, ci, ci, vp, ci]
    lib.stz_mg_level_gs_colours.argtypes = [vp, ci, ci, ci]
    lib.stz_mg_level_restrict_residual.argtypes = [vp, ci]
    lib.stz_mg_level_interpolation.argtypes = [vp, ci]
    lib.stz_mg_level_residual.argtypes = [vp, ci, vp, ctypes.POINTER(cd), ci]
    lib.stz_mg_time_kernel.argtypes = [vp, ci, ci, ci, ctypes.POINTER(cd), ctypes.POINTER(cd)]
    lib.stz_mg_sweep_kind.argtypes = [vp, ci, ctypes.POINTER(ci), ctypes.POINTER(ci)]
    lib.stz_mg_const_residual_sumsq_noalloc.argtypes = [ci, ci, ci, ci, ci, ci, vp, vp, vp, vp, vp, ci, vp]
    lib.stz_mg_adjoint_solve.argtypes = [vp, vp, vp, ci, cd, ci, ctypes.POINTER(ci), ctypes.POINTER(cd)]
    lib.stz_mg_coeff_grad.argtypes = [vp, vp, vp, vp, vp, ci]
    lib.stz_mg_stress_update.argtypes = [vp, vp, cd, cd, cd, cd, cd, cd, ctypes.POINTER(cd), ci]
    lib.stz_mg_advection_step.argtypes = [vp, vp, cd, vp, ctypes.POINTER(ci)]
    lib.stz_mg_output_slice.argtypes = [vp, ci, ci, cd, cd, cd, cd, ctypes.c_char_p]
    lib.stz_mg_cube_values.argtypes = [vp, ci, ci, ci, ci, vp, vp]
    lib.stz_mg_output_cube.argtypes = [vp, ci, ci, ci, ci, ctypes.c_char_p, ctypes.c_char_p, ci]
    for name in EXPORTS:
        if name not in ("stz_mg_desc_default", "stz_mg_last_error"):
            getattr(lib, name).restype = ci
    _lib = lib
    return lib


def _check(rc):
    if rc != OK:
        raise StzMgError(rc, load_library().stz_mg_last_error().decode())


def _arg(a, n=None):
    """(pointer, where) of a float64 array: numpy (host) or CUDA torch tensor."""
    if hasattr(a, "data_ptr") and hasattr(a, "is_cuda"):
        import torch
        if a.dtype != torch.float64 or not a.is_contiguous():
            raise ValueError("device arrays must be contiguous float64 tensors")
        if n is not None and a.numel() != n:
            raise ValueError(f"expected {n} elements, got {a.numel()}")
        if a.is_cuda:
            # the handle's stream reads or writes this memory: torch's work on
            # it (producing an input, or still reading a recycled output
            # block) must be finished first
            torch.cuda.current_stream(a.device).synchronize()
            return ctypes.c_void_p(a.data_ptr()), DEVICE, a
        a = a.numpy()
    arr = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and arr.size != n:
        raise ValueError(f"expected {n} elements, got {arr.size}")
    return arr.ctypes.data_as(ctypes.c_void_p), HOST, arr


def elastic_stencil(mu, lam, dx, dy, dz, dt=1.0):
    """27x9 stencil and 3x3 fix block of the constant-coefficient operator.

    Host helper mirroring shear_sim_3d::set_up_stencil_base
    (src/shear_sim_3d.cpp:215-331, kappa = 0) and
    set_up_stencil_and_matrices (src/shear_sim_3d.hh:45-55): the negated,
    dt-scaled discretisation of (lam+2mu) u_xx + mu (u_yy + u_zz) +
    (lam+mu)(v_xy + w_xz) and its permutations.
    """
    base = np.zeros((3, 3, 3, 3, 3))   # [dz+1, dy+1, dx+1, row, col]
    lm = (lam + mu)
    h = (dx, dy, dz)
    for ax in range(3):
        for s in (-1, 1):
            d = [1, 1, 1]
            d[ax] = 1 + s
            diag = [mu / h[ax] / h[ax]] * 3
            diag[ax] = (lam + 2 * mu) / h[ax] / h[ax]
            base[d[2], d[1], d[0]] = np.diag(diag)
    base[1, 1, 1] = -np.diag([2 * ((lam + 2 * mu) / dx / dx + mu / dy / dy + mu / dz / dz),
                              2 * (mu / dx / dx + (lam + 2 * mu) / dy / dy + mu / dz / dz),
                              2 * (mu / dx / dx + mu / dy / dy + (lam + 2 * mu) / dz / dz)])
    for (r, c) in ((0, 1), (0, 2), (1, 2)):
        for sr in (-1, 1):
            for sc in (-1, 1):
                d = [1, 1, 1]
                d[r] += sr
                d[c] += sc
                v = sr * sc * lm / 4 / h[r] / h[c]
                base[d[2], d[1], d[0], r, c] = v
                base[d[2], d[1], d[0], c, r] = v
    stencil = (-dt * base).reshape(27, 9)
    fix = np.eye(3).reshape(9) * (-dt * 2 * ((lam + 2 * mu) / dx / dx + mu / dy / dy + mu / dz / dz))
    return stencil, fix


class Multigrid:
    """GPU multigrid<vec3, mat3> for one problem on one device.

    Parameters mirror the reference: grid size and periodicity (region ctor),
    v_down/v_up (multigrid.hh:24-32), and the hierarchy stop rule
    ``max_coarse`` (reference: 1024).  ``precision`` is "fp64" or "mixed"
    (FP32 V-cycles inside FP64 defect correction); ``bottom`` is "direct"
    (FP64 dense solve of the coarsest level) or "gs" (``bottom_sweeps``
    Gauss-Seidel sweeps, the reference's solve_exact).  ``sweep_growth`` keeps
    the reference's 2+i sweeps on level i; False uses v_down/v_up everywhere."""

    def __init__(self, dims, periodic=(True, True, False), precision="fp64", v_down=2, v_up=2,
                 max_coarse=1024, bottom="direct", bottom_sweeps=24, sweep_growth=True, device=0, stream=None):
        lib = load_library()
        d = Desc()
        lib.stz_mg_desc_default(ctypes.byref(d))
        d.m, d.n, d.o = (int(v) for v in dims)
        d.x_prd, d.y_prd, d.z_prd = (int(bool(p)) for p in periodic)
        d.precision = {"fp64": FP64, "mixed": MIXED}[precision]
        d.v_down, d.v_up = v_down, v_up
        d.max_coarse = max_coarse
        d.bottom = {"direct": BOTTOM_DIRECT, "gs": BOTTOM_GS}[bottom]
        d.bottom_sweeps = bottom_sweeps
        d.sweep_growth = int(bool(sweep_growth))
        d.device = device
        d.stream = stream
        self.dims = tuple(int(v) for v in dims)
        self.periodic = tuple(bool(p) for p in periodic)
        self.precision = precision
        h = ctypes.c_void_p()
        _check(lib.stz_mg_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h

    # ---------------------------------------------------------------- life
    def close(self):
        if getattr(self, "_h", None):
            load_library().stz_mg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def npts(self):
        m, n, o = self.dims
        return m * n * o

    # ----------------------------------------------------------- operators
    def set_stencil_const(self, stencil, fix):
        st, _, a = _arg(np.asarray(stencil, dtype=np.float64).reshape(243), 243)
        fx, _, b = _arg(np.asarray(fix, dtype=np.float64).reshape(9), 9)
        _check(load_library().stz_mg_set_stencil_const(self._h, st, fx))

    def set_stencil_points(self, A):
        p, where, keep = _arg(A, 243 * self.npts)
        _check(load_library().stz_mg_set_stencil_points(self._h, p, where))

    def set_coeffs_lame(self, mu, lam, dx, dy, dz, dt=1.0):
        pm, wm, k1 = _arg(mu, self.npts)
        pl, wl, k2 = _arg(lam, self.npts)
        if wm != wl:
            raise ValueError("mu and lam must both be host or both be device arrays")
        _check(load_library().stz_mg_set_coeffs_lame(self._h, pm, pl, dx, dy, dz, dt, wm))

    def setup_matrices(self, stencil=None, fix=None, points=None, mu=None, lam=None, spacing=None, dt=1.0):
        """multigrid::setup_matrices: top-level operator, then RAT on every level."""
        if stencil is not None:
            self.set_stencil_const(stencil, fix)
        elif points is not None:
            self.set_stencil_points(points)
        elif mu is not None:
            self.set_coeffs_lame(mu, lam, *spacing, dt=dt)
        _check(load_library().stz_mg_setup(self._h))

    # -------------------------------------------------------------- fields
    def set_rhs(self, r):
        p, where, keep = _arg(r, 3 * self.npts)
        _check(load_library().stz_mg_set_rhs(self._h, p, where))

    def set_x(self, x):
        p, where, keep = _arg(x, 3 * self.npts)
        _check(load_library().stz_mg_set_x(self._h, p, where))

    def setup_fields(self, x=None, r=None):
        """multigrid::setup_fields: initial guess (zero when None) and right-hand side."""
        self.set_x(np.zeros(3 * self.npts) if x is None else x)
        if r is not None:
            self.set_rhs(r)

    def set_rhs_divergence(self, eps, spacing):
        """Right-hand side = node divergence of the cell tensor field eps
        (6 components per cell), assembled on the device."""
        m, n, o = self.dims
        xp, yp, zp = self.periodic
        ncells = (m if xp else m - 1) * (n if yp else n - 1) * (o if zp else o - 1)
        p, where, keep = _arg(eps, 6 * ncells)
        _check(load_library().stz_mg_set_rhs_divergence(self._h, p, *spacing, where))

    def get_rhs(self, out=None):
        if out is None:
            out = np.empty((self.npts, 3))
        p, where, keep = _arg(out, 3 * self.npts)
        _check(load_library().stz_mg_get_rhs(self._h, p, where))
        return out

    def get_x(self, out=None):
        if out is None:
            out = np.empty((self.npts, 3))
        p, where, keep = _arg(out, 3 * self.npts)
        _check(load_library().stz_mg_get_x(self._h, p, where))
        return out

    def stress_update(self, sigma, lam, mu, dt, spacing):
        """Projection-step stress update (shear_sim_3d.cpp:681-710) from the
        current solution: sigma (6 per cell, a float64 numpy array or CUDA
        tensor) is updated in place; returns proj_mag."""
        m, n, o = self.dims
        xp, yp, zp = self.periodic
        ncells = (m if xp else m - 1) * (n if yp else n - 1) * (o if zp else o - 1)
        if hasattr(sigma, "is_cuda") and sigma.is_cuda:
            p, where, keep = _arg(sigma, 6 * ncells)
        else:
            if not (isinstance(sigma, np.ndarray) and sigma.dtype == np.float64 and sigma.flags.c_contiguous):
                raise ValueError("sigma must be a contiguous float64 array (updated in place)")
            if sigma.size != 6 * ncells:
                raise ValueError(f"expected {6 * ncells} elements, got {sigma.size}")
            p, where = sigma.ctypes.data_as(ctypes.c_void_p), HOST
        pm = ctypes.c_double()
        _check(load_library().stz_mg_stress_update(self._h, p, lam, mu, dt, *spacing, ctypes.byref(pm), where))
        return pm.value

    # --------------------------------------------------------------- solve
    def v_cycle(self):
        _check(load_library().stz_mg_vcycle(self._h))

    def solve(self, tol=1e-10, max_cycles=100, check=True):
        """V-cycles until |b-Ax|/|b| <= tol.  Returns (cycles, relres)."""
        c, r = ctypes.c_int(), ctypes.c_double()
        rc = load_library().stz_mg_solve(self._h, tol, max_cycles, ctypes.byref(c), ctypes.byref(r))
        if rc != OK and (check or rc != ERR_NOCONV):
            _check(rc)
        return c.value, r.value

    def solve_stats(self):
        """(V-cycles, top-level residual evaluations, kernels launched) of the last solve."""
        c, r, k = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        _check(load_library().stz_mg_solve_stats(self._h, ctypes.byref(c), ctypes.byref(r), ctypes.byref(k)))
        return c.value, r.value, k.value

    def residual_norm(self):
        rn, bn = ctypes.c_double(), ctypes.c_double()
        _check(load_library().stz_mg_residual_norm(self._h, ctypes.byref(rn), ctypes.byref(bn)))
        return rn.value, bn.value

    def l2_error_all(self):
        """region::l2_error_all as shipped (sum of |r|^4 for vec3)."""
        v = ctypes.c_double()
        _check(load_library().stz_mg_l2_error_all(self._h, ctypes.byref(v)))
        return v.value

    # ------------------------------------------------------------- adjoint
    def adjoint_solve(self, g, out=None, tol=1e-10, max_cycles=100):
        """w with A^T w = g (overwrites the handle's x and right-hand side).
        Returns (w, cycles, relres)."""
        pg, wg, keep = _arg(g, 3 * self.npts)
        if out is None:
            if wg == DEVICE:
                import torch
                out = torch.empty_like(g)
            else:
                out = np.empty((self.npts, 3))
        po, wo, keep2 = _arg(out, 3 * self.npts)
        if wo != wg:
            raise ValueError("g and out must both be host or both be device arrays")
        c, r = ctypes.c_int(), ctypes.c_double()
        _check(load_library().stz_mg_adjoint_solve(self._h, pg, po, wg, tol, max_cycles, ctypes.byref(c),
                                                   ctypes.byref(r)))
        return out, c.value, r.value

    def coeff_grad(self, w, u, dmu=None, dlam=None):
        """(-w^T dA/dmu u, -w^T dA/dlam u) per node of the Lame operator."""
        pw, ww, k1 = _arg(w, 3 * self.npts)
        pu, wu, k2 = _arg(u, 3 * self.npts)
        if ww != wu:
            raise ValueError("w and u must both be host or both be device arrays")
        if dmu is None:
            if ww == DEVICE:
                import torch
                dmu = torch.empty(self.npts, dtype=torch.float64, device=w.device)
                dlam = torch.empty(self.npts, dtype=torch.float64, device=w.device)
            else:
                dmu, dlam = np.empty(self.npts), np.empty(self.npts)
        pm, wm, k3 = _arg(dmu, self.npts)
        pl, wl, k4 = _arg(dlam, self.npts)
        if not (wm == wl == ww):
            raise ValueError("all arrays must be on the same side")
        _check(load_library().stz_mg_coeff_grad(self._h, pw, pu, pm, pl, ww))
        return dmu, dlam

    # -------------------------------------------------------------- levels
    @property
    def nlevels(self):
        v = ctypes.c_int()
        _check(load_library().stz_mg_num_levels(self._h, ctypes.byref(v)))
        return v.value

    def level_dims(self, l):
        d = np.zeros(3, dtype=np.int32)
        _check(load_library().stz_mg_level_dims(self._h, l, d.ctypes.data_as(ctypes.c_void_p)))
        return tuple(int(v) for v in d)

    def level_npts(self, l):
        m, n, o = self.level_dims(l)
        return m * n * o

    def level_operator(self, l):
        N = self.level_npts(l)
        A = np.zeros((N, 27, 9))
        S = np.zeros((N, 6), dtype=np.int32)
        _check(load_library().stz_mg_level_operator(self._h, l, A.ctypes.data_as(ctypes.c_void_p),
                                                    S.ctypes.data_as(ctypes.c_void_p)))
        return A, S

    def level_set_field(self, l, which, v):
        p, where, keep = _arg(v, 3 * self.level_npts(l))
        _check(load_library().stz_mg_level_set_field(self._h, l, _FIELDS[which], p, where))

    def level_get_field(self, l, which):
        out = np.empty((self.level_npts(l), 3))
        _check(load_library().stz_mg_level_get_field(self._h, l, _FIELDS[which],
                                                     out.ctypes.data_as(ctypes.c_void_p), HOST))
        return out

    def level_get_planes(self, l, which, k0, nk, out=None):
        """z-planes k0 .. k0+nk-1 of field `which` ("x", "r", "res") of level l,
        (nk*m*n, 3) in natural order: a numpy array, or written into `out`
        (a numpy array or a float64 CUDA tensor)."""
        m, n, _ = self.level_dims(l)
        if out is None:
            out = np.empty((nk * m * n, 3))
        p, where, keep = _arg(out, 3 * m * n * nk)
        _check(load_library().stz_mg_level_get_planes(self._h, l, _FIELDS[which], k0, nk, p, where))
        return out

    def level_set_planes(self, l, which, k0, v):
        """Set z-planes k0 .. of field `which` of level l from (nk*m*n, 3) values."""
        m, n, _ = self.level_dims(l)
        nk = (v.numel() if hasattr(v, "numel") else np.size(v)) // (3 * m * n)
        p, where, keep = _arg(v, 3 * m * n * nk)
        _check(load_library().stz_mg_level_set_planes(self._h, l, _FIELDS[which], k0, nk, p, where))

    def gauss_seidel_colours(self, l, q0, q1):
        """Colour passes q0 .. q1-1 of the 8-colour sweep of level l (FP64)."""
        _check(load_library().stz_mg_level_gs_colours(self._h, l, q0, q1))

    def restrict_residual(self, l):
        """Coarse r of level l from the level-(l-1) residual field as it stands; coarse x = 0."""
        _check(load_library().stz_mg_level_restrict_residual(self._h, l))

    def gauss_seidel(self, l, sweeps=1):
        _check(load_library().stz_mg_level_gauss_seidel(self._h, l, sweeps))

    def restriction(self, l):
        _check(load_library().stz_mg_level_restriction(self._h, l))

    def interpolation(self, l):
        _check(load_library().stz_mg_level_interpolation(self._h, l))

    def compute_residual(self, l=0):
        """r - A x of level l into its residual field (STZ_MG_FIELD_RES),
        nothing copied out; returns |r - A x|^2."""
        sq = ctypes.c_double()
        _check(load_library().stz_mg_level_residual(self._h, l, None, ctypes.byref(sq), HOST))
        return sq.value

    def residual(self, l=0):
        out = np.empty((self.level_npts(l), 3))
        sq = ctypes.c_double()
        _check(load_library().stz_mg_level_residual(self._h, l, out.ctypes.data_as(ctypes.c_void_p),
                                                    ctypes.byref(sq), HOST))
        return out, sq.value

    def output_slice(self, which, k, filename, box=None):
        """region::output_x / output_r / output_residual: the z-slice k of the
        solution ("x"), right-hand side ("r") or residual ("residual") written
        to filename in the reference's slice format; box = (ax, bx, ay, by),
        default (0, m-1, 0, n-1)."""
        m, n, _ = self.dims
        ax, bx, ay, by = box if box is not None else (0.0, m - 1.0, 0.0, n - 1.0)
        code = {"x": 0, "r": 1, "residual": 2}[which]
        _check(load_library().stz_mg_output_slice(self._h, code, k, ax, bx, ay, by, os.fsencode(filename)))

    def sweep_kind(self, level=0):
        """(kind, launches per sweep) of the smoother of a level: kind is one
        of "colour", "tile", "band", "phase"."""
        k, n = ctypes.c_int(), ctypes.c_int()
        _check(load_library().stz_mg_sweep_kind(self._h, level, ctypes.byref(k), ctypes.byref(n)))
        return ("colour", "tile", "band", "phase")[k.value], n.value

    def time_kernel(self, kernel, level=0, reps=20):
        """(ms per launch, algorithmic bytes or FP64 flops per launch) of one
        solver kernel, timed with CUDA events on the handle's stream."""
        ms, work = ctypes.c_double(), ctypes.c_double()
        _check(load_library().stz_mg_time_kernel(self._h, kernel, level, reps, ctypes.byref(ms), ctypes.byref(work)))
        return ms.value, work.value
