"""ctypes wrapper of the compiled reference multigrid (oracle/_ref/libstzref.so).

Test infrastructure only.  The library is the reference's own mg_3d_template
sources compiled with the single-rank MPI shim (oracle/Makefile, target
``ref``); it exists only where the reference checkout was available at build
time, so callers must handle :func:`available` being False.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libstzref.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(LIB_PATH)
    lib.sr_last_error.restype = ctypes.c_char_p
    lib.sr_create.argtypes = [ctypes.c_int] * 6 + [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    lib.sr_destroy.argtypes = [ctypes.c_void_p]
    lib.sr_num_levels.argtypes = [ctypes.c_void_p]
    for name in ("sr_level_dims", "sr_level_S"):
        getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.sr_level_A.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.sr_set_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.sr_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.sr_gauss_seidel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.sr_restriction.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.sr_interpolation.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.sr_vcycle.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.sr_residual.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.sr_l2_error_all.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.sr_solve.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.sr_output_slice.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int] + \
        [ctypes.c_double] * 4 + [ctypes.c_char_p]
    _lib = lib
    return lib


def available() -> bool:
    return os.path.exists(LIB_PATH)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class RefMultigrid:
    """The reference multigrid<vec3,mat3> on one rank.

    ``max_coarse`` is the coarsest-level size rule: the reference coarsens
    while total() > 1024 (multigrid.cc:40); smaller values extend the
    hierarchy with further reference regions."""

    def __init__(self, dims, periodic, stencil=None, fix=None, points=None, max_coarse=1024):
        lib = _load()
        m, n, o = dims
        self.dims = (m, n, o)
        self.periodic = tuple(bool(p) for p in periodic)
        st = None if stencil is None else np.ascontiguousarray(stencil, dtype=np.float64).reshape(27 * 9)
        fx = None if fix is None else np.ascontiguousarray(fix, dtype=np.float64).reshape(9)
        pts = None if points is None else np.ascontiguousarray(points, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = lib.sr_create(m, n, o, *[int(p) for p in periodic], _ptr(st), _ptr(fx), _ptr(pts),
                           int(max_coarse), ctypes.byref(h))
        self._check(rc)
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference oracle: " + _load().sr_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            _load().sr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nlevels(self):
        return _load().sr_num_levels(self._h)

    def level_dims(self, l):
        d = np.zeros(3, dtype=np.int32)
        self._check(_load().sr_level_dims(self._h, l, _ptr(d)))
        return tuple(int(v) for v in d)

    def npts(self, l):
        m, n, o = self.level_dims(l)
        return m * n * o

    def level_S(self, l):
        S = np.zeros((self.npts(l), 6), dtype=np.int32)
        self._check(_load().sr_level_S(self._h, l, _ptr(S)))
        return S

    def level_A(self, l):
        A = np.zeros((self.npts(l), 27, 9))
        self._check(_load().sr_level_A(self._h, l, _ptr(A)))
        return A

    def set_field(self, l, which, v):
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(self.npts(l), 3)
        self._check(_load().sr_set_field(self._h, l, {"x": 0, "r": 1}[which], _ptr(v)))

    def output_slice(self, which, k, box, filename, l=0):
        """region::output_x / output_r / output_residual (which: "x", "r",
        "residual") of level l: z-slice k in box (ax, bx, ay, by) to filename."""
        self._check(_load().sr_output_slice(self._h, l, {"x": 0, "r": 1, "residual": 2}[which], k, *box,
                                            filename.encode()))

    def get_field(self, l, which):
        v = np.zeros((self.npts(l), 3))
        self._check(_load().sr_get_field(self._h, l, {"x": 0, "r": 1}[which], _ptr(v)))
        return v

    def gauss_seidel(self, l, sweeps=1):
        self._check(_load().sr_gauss_seidel(self._h, l, sweeps))

    def restriction(self, l):
        self._check(_load().sr_restriction(self._h, l))

    def interpolation(self, l):
        self._check(_load().sr_interpolation(self._h, l))

    def v_cycle(self, bottom="gs"):
        self._check(_load().sr_vcycle(self._h, {"gs": 0, "direct": 1}[bottom]))

    def residual(self, l=0):
        out = np.zeros((self.npts(l), 3))
        sq = ctypes.c_double()
        self._check(_load().sr_residual(self._h, l, _ptr(out), ctypes.byref(sq)))
        return out, sq.value

    def l2_error_all(self, l=0):
        v = ctypes.c_double()
        self._check(_load().sr_l2_error_all(self._h, l, ctypes.byref(v)))
        return v.value

    def solve(self, tol=1e-10, max_cycles=100, bottom="gs"):
        hist = np.zeros(max_cycles)
        c = ctypes.c_int()
        self._check(_load().sr_solve(self._h, tol, max_cycles, {"gs": 0, "direct": 1}[bottom],
                                     ctypes.byref(c), _ptr(hist)))
        return c.value, hist[: c.value]
