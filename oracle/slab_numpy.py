"""numpy sub-domains for the CPU tests of the z-slab decomposition.

Test infrastructure only: a plain numpy level (x, r, res and one coarse
level) with the operations the decomposition drives -- 8-colour
Gauss-Seidel passes of a shared stencil (region::gauss_seidel,
mg_3d_template/region.cc:1557-1762, in the colour order), the residual
(region.cc:1008-1055), full-weighting restriction and trilinear
interpolation with the regular weights (region.cc:2129-2186, 2061-2121;
coarse planes whose fine neighbours fall outside a non-periodic z are left
at zero) -- with the interface of stzpp_gb300.slabs.HandleSlab.  The same
class serves as the undivided reference (the whole grid, z periodic or not)
and as one slab (its planes and ghosts, z not periodic), so the CPU tests
check the decomposition's exchanges and transfers, not the GPU kernels.
The grid is periodic in x and y.
"""
from __future__ import annotations

import numpy as np

_OFF = [((b % 3) - 1, ((b // 3) % 3) - 1, (b // 9) - 1) for b in range(27)]


class NumpyLevel:
    def __init__(self, m, n, o, zp, stencil, fix):
        self.m, self.n, self.o, self.zp = m, n, o, zp
        self.A = np.asarray(stencil, dtype=np.float64).reshape(27, 3, 3)
        self.F = np.asarray(fix, dtype=np.float64).reshape(3, 3)
        self.inv_int = np.linalg.inv(self.A[13])
        self.inv_fix = np.linalg.inv(self.F)
        self.f = {w: np.zeros((o, n, m, 3)) for w in ("x", "r", "res")}
        self.mc, self.nc, self.oc = m // 2, n // 2, (o + (1 if zp else 2)) >> 1
        self.cf = {w: np.zeros((self.oc, self.nc, self.mc, 3)) for w in ("x", "r")}

    # ------------------------------------------------------- interface
    def plane_size(self, level):
        return self.m * self.n if level == 0 else self.mc * self.nc

    def nplanes(self, level):
        return self.o if level == 0 else self.oc

    def empty_planes(self, level, nk):
        return np.empty((nk * self.plane_size(level), 3))

    def _field(self, level, which):
        return self.f[which] if level == 0 else self.cf[which]

    def get_planes(self, level, which, k0, nk):
        return self._field(level, which)[k0:k0 + nk].reshape(-1, 3).copy()

    def set_planes(self, level, which, k0, v):
        f = self._field(level, which)
        nk = v.shape[0] // self.plane_size(level)
        f[k0:k0 + nk] = np.asarray(v).reshape((nk,) + f.shape[1:])

    def _nodes(self, q):
        a, b, c = q & 1, (q >> 1) & 1, q >> 2
        return np.meshgrid(np.arange(c, self.o, 2), np.arange(b, self.n, 2), np.arange(a, self.m, 2), indexing="ij")

    def _interior(self, K):
        return np.ones(K.shape, bool) if self.zp else (K != 0) & (K != self.o - 1)

    def _apply(self, K, J, I, with_centre):
        """sum over the box of A_b x_b at nodes (K, J, I), block order."""
        x = self.f["x"]
        acc = np.zeros(K.shape + (3,))
        for b, (dx, dy, dz) in enumerate(_OFF):
            if b == 13 and not with_centre:
                continue
            kk = K + dz
            if self.zp:
                kk = kk % self.o
            kk = np.clip(kk, 0, self.o - 1)
            v = x[kk, (J + dy) % self.n, (I + dx) % self.m]
            a = self.A[b]
            acc = acc + np.stack([(a[r, 0] * v[..., 0] + a[r, 1] * v[..., 1]) + a[r, 2] * v[..., 2]
                                  for r in range(3)], axis=-1)
        return acc

    @staticmethod
    def _mv(M, v):
        return np.stack([(M[r, 0] * v[..., 0] + M[r, 1] * v[..., 1]) + M[r, 2] * v[..., 2] for r in range(3)], axis=-1)

    def colours(self, q0, q1):
        x, r = self.f["x"], self.f["r"]
        for q in range(q0, q1):
            K, J, I = self._nodes(q)
            if K.size == 0:
                continue
            inner = self._interior(K)
            d = r[K, J, I] - self._apply(K, J, I, False)
            new = np.where(inner[..., None], self._mv(self.inv_int, d), self._mv(self.inv_fix, r[K, J, I]))
            x[K, J, I] = new

    def residual(self):
        K, J, I = np.meshgrid(np.arange(self.o), np.arange(self.n), np.arange(self.m), indexing="ij")
        inner = self._interior(K)
        full = self.f["r"] - self._apply(K, J, I, True)
        plate = self.f["r"] - self._mv(self.F, self.f["x"])
        self.f["res"] = np.where(inner[..., None], full, plate)

    def sumsq_planes(self, level, which, k0, nk):
        v = self._field(level, which)[k0:k0 + nk]
        return float((v * v).sum())

    def restrict(self):
        res = self.f["res"]
        out = np.zeros_like(self.cf["r"])
        Kc = np.arange(self.oc)
        for dz in (-1, 0, 1):
            kf = 2 * Kc + dz
            ok = np.ones(Kc.shape, bool) if self.zp else (kf >= 0) & (kf < self.o)
            if self.zp:
                kf = kf % self.o
            for dy in (-1, 0, 1):
                jf = (2 * np.arange(self.nc) + dy) % self.n
                for dx in (-1, 0, 1):
                    i_f = (2 * np.arange(self.mc) + dx) % self.m
                    w = 0.125 * 0.5 ** ((dx != 0) + (dy != 0) + (dz != 0))
                    blk = res[np.ix_(np.clip(kf, 0, self.o - 1), jf, i_f)] * w
                    out += np.where(ok[:, None, None, None], blk, 0.0)
        if not self.zp:   # coarse planes reaching past the ends are not the regular formula's
            bad = (2 * Kc - 1 < 0) | (2 * Kc + 1 > self.o - 1)
            out[bad] = 0.0
        self.cf["r"] = out
        self.cf["x"] = np.zeros_like(out)

    def interpolate(self):
        xc = self.cf["x"]
        x = self.f["x"]

        def parents(f, nf, nc, prd):
            if f % 2 == 0:
                return [(f // 2, 1.0)]
            ps = [((f - 1) // 2, 0.5), ((f + 1) // 2, 0.5)]
            return [((p % nc) if prd else p, w) for p, w in ps]

        for k in range(self.o):
            pk = parents(k, self.o, self.oc, self.zp)
            if any(p < 0 or p >= self.oc for p, _ in pk):
                continue
            for j in range(self.n):
                pj = parents(j, self.n, self.nc, True)
                for i in range(self.m):
                    pi = parents(i, self.m, self.mc, True)
                    s = np.zeros(3)
                    for a, wa in pk:
                        for b, wb in pj:
                            for c, wc in pi:
                                s = s + (wa * wb * wc) * xc[a, b, c]
                    x[k, j, i] = x[k, j, i] + s
