"""ctypes wrapper of the C restatement of the reference multigrid
(oracle/stzmg_oracle.c, built as oracle/liboracle.so).

Test infrastructure only: the oracle that the GPU tests, ``smoke()`` and the
bench's CPU leg compare against.  It is built from this repository's own
sources on every machine (``make -C oracle port``), unlike the compiled
reference in ``oracle/_ref``.  Same interface as :class:`oracle.refpy.RefMultigrid`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

SMOOTHERS = {"lex": 0, "mc8": 1}
BOTTOMS = {"gs": 0, "direct": 1}


def _load():
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(LIB_PATH)
    vp, ci = ctypes.c_void_p, ctypes.c_int
    lib.so_last_error.restype = ctypes.c_char_p
    lib.so_create.argtypes = [ci] * 6 + [vp] * 3 + [ci, ctypes.POINTER(vp)]
    lib.so_destroy.argtypes = [vp]
    lib.so_num_levels.argtypes = [vp]
    for name in ("so_level_dims", "so_level_S", "so_level_A"):
        getattr(lib, name).argtypes = [vp, ci, vp]
    lib.so_set_field.argtypes = [vp, ci, ci, vp]
    lib.so_get_field.argtypes = [vp, ci, ci, vp]
    lib.so_gauss_seidel.argtypes = [vp, ci, ci, ci]
    lib.so_restriction.argtypes = [vp, ci]
    lib.so_interpolation.argtypes = [vp, ci]
    lib.so_vcycle.argtypes = [vp, ci, ci]
    lib.so_residual.argtypes = [vp, ci, vp, vp]
    lib.so_solve.argtypes = [vp, ctypes.c_double, ci, ci, ci, vp, vp]
    lib.so_set_cycle.argtypes = [vp, ci, ci, ci, ci]
    lib.so_set_threads.argtypes = [ci]
    lib.so_threads.restype = ci
    _lib = lib
    return lib


def set_threads(n: int) -> int:
    """Host threads of every handle (1: the serial restatement; P > 1: the
    reference's z-decomposed sweep on P slabs).  Returns the count in effect."""
    lib = _load()
    lib.so_set_threads(int(n))
    return lib.so_threads()


def available() -> bool:
    return os.path.exists(LIB_PATH)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class PortMultigrid:
    """The restated multigrid<vec3,mat3> (see oracle/stzmg_oracle.h)."""

    def __init__(self, dims, periodic, stencil=None, fix=None, points=None, max_coarse=1024):
        lib = _load()
        m, n, o = dims
        self.dims = (m, n, o)
        self.periodic = tuple(bool(p) for p in periodic)
        st = None if stencil is None else np.ascontiguousarray(stencil, dtype=np.float64).reshape(243)
        fx = None if fix is None else np.ascontiguousarray(fix, dtype=np.float64).reshape(9)
        pts = None if points is None else np.ascontiguousarray(points, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = lib.so_create(m, n, o, *[int(p) for p in periodic], _ptr(st), _ptr(fx), _ptr(pts),
                           int(max_coarse), ctypes.byref(h))
        self._check(rc)
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + _load().so_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            _load().so_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nlevels(self):
        return _load().so_num_levels(self._h)

    def level_dims(self, l):
        d = np.zeros(3, dtype=np.int32)
        self._check(_load().so_level_dims(self._h, l, _ptr(d)))
        return tuple(int(v) for v in d)

    def npts(self, l):
        m, n, o = self.level_dims(l)
        return m * n * o

    def level_S(self, l):
        S = np.zeros((self.npts(l), 6), dtype=np.int32)
        self._check(_load().so_level_S(self._h, l, _ptr(S)))
        return S

    def level_A(self, l):
        A = np.zeros((self.npts(l), 27, 9))
        self._check(_load().so_level_A(self._h, l, _ptr(A)))
        return A

    def set_field(self, l, which, v):
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(self.npts(l), 3)
        self._check(_load().so_set_field(self._h, l, {"x": 0, "r": 1}[which], _ptr(v)))

    def get_field(self, l, which):
        v = np.zeros((self.npts(l), 3))
        self._check(_load().so_get_field(self._h, l, {"x": 0, "r": 1}[which], _ptr(v)))
        return v

    def set_cycle(self, v_down=2, v_up=2, bottom_sweeps=24, grow=True):
        self._check(_load().so_set_cycle(self._h, v_down, v_up, bottom_sweeps, int(grow)))

    def gauss_seidel(self, l, sweeps=1, smoother="lex"):
        self._check(_load().so_gauss_seidel(self._h, l, sweeps, SMOOTHERS[smoother]))

    def restriction(self, l):
        self._check(_load().so_restriction(self._h, l))

    def interpolation(self, l):
        self._check(_load().so_interpolation(self._h, l))

    def v_cycle(self, bottom="gs", smoother="lex"):
        self._check(_load().so_vcycle(self._h, SMOOTHERS[smoother], BOTTOMS[bottom]))

    def residual(self, l=0):
        out = np.zeros((self.npts(l), 3))
        sq = ctypes.c_double()
        self._check(_load().so_residual(self._h, l, _ptr(out), ctypes.byref(sq)))
        return out, sq.value

    def residual_sq(self, l=0):
        """|r - A x|^2 of level l without copying the residual out."""
        sq = ctypes.c_double()
        self._check(_load().so_residual(self._h, l, None, ctypes.byref(sq)))
        return sq.value

    def solve(self, tol=1e-10, max_cycles=100, bottom="gs", smoother="lex"):
        hist = np.zeros(max_cycles)
        c = ctypes.c_int()
        self._check(_load().so_solve(self._h, tol, max_cycles, SMOOTHERS[smoother], BOTTOMS[bottom],
                                     ctypes.byref(c), _ptr(hist)))
        return c.value, hist[: c.value]
