"""Oracle of the adjoint of the projection solve (test infrastructure only).

For u = A(mu, lam)^{-1} b and a scalar loss L(u) with g = dL/du:
    dL/db = w,  A^T w = g,
    dL/dmu_q = -w^T (dA/dmu_q) u,  dL/dlam_q = -w^T (dA/dlam_q) u.
Everything here is computed from the oracle's own operator
(problem.elastic_stencil_points, the per-node stencils the reference's
fill_entries path would receive) with scipy sparse direct solves, and the
coefficient derivatives by LINEARITY of the operator in (mu, lam): no
derivative formula is restated.  Probing uses colour classes of nodes 4 apart
in every dimension, so that no row of A depends on two nodes of one class
(a row uses mu, lam only at its node and its 6 face neighbours).

The reference has no adjoint (its solver is not differentiated); this oracle
is pinned by the definition above and by finite differences in the tests.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import problem as P


def assemble(points, dims, periodic):
    """Sparse 3N x 3N matrix of per-node stencils (npts, 27, 9), natural order."""
    m, n, o = dims
    N = m * n * o
    pts = points.reshape(N, 27, 3, 3)
    k, j, i = np.meshgrid(np.arange(o), np.arange(n), np.arange(m), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    rows, cols, vals = [], [], []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                b = P.block_index(dx, dy, dz)
                ii, jj, kk = i + dx, j + dy, k + dz
                ok = np.ones(N, dtype=bool)
                for a, L, per in ((ii, m, periodic[0]), (jj, n, periodic[1]), (kk, o, periodic[2])):
                    if per:
                        a %= L
                    else:
                        ok &= (a >= 0) & (a < L)
                q = ii + m * (jj + n * kk)
                blk = pts[:, b]
                nz = ok & np.any(blk != 0, axis=(1, 2))
                p_idx = np.nonzero(nz)[0]
                for r in range(3):
                    for c in range(3):
                        v = blk[p_idx, r, c]
                        keep = v != 0
                        rows.append(3 * p_idx[keep] + r)
                        cols.append(3 * q[p_idx[keep]] + c)
                        vals.append(v[keep])
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(3 * N, 3 * N))
    A.sum_duplicates()
    return A


def solve(A, rhs):
    return spla.spsolve(A.tocsc(), rhs.reshape(-1)).reshape(-1, 3)


def _class_period(L, per):
    return 4 if (not per or L % 4 == 0) else L


def neighbours(dims, periodic):
    """(N, 27) natural index of each node's neighbour at block b (0 where it
    leaves a non-periodic grid; the coefficients there are zero)."""
    m, n, o = dims
    k, j, i = np.meshgrid(np.arange(o), np.arange(n), np.arange(m), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    nb = np.zeros((m * n * o, 27), dtype=np.int64)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                ii, jj, kk = i + dx, j + dy, k + dz
                ok = np.ones(ii.shape, dtype=bool)
                for a, L, per in ((ii, m, periodic[0]), (jj, n, periodic[1]), (kk, o, periodic[2])):
                    if per:
                        a %= L
                    else:
                        ok &= (a >= 0) & (a < L)
                nb[:, P.block_index(dx, dy, dz)] = np.where(ok, ii + m * (jj + n * kk), 0)
    return nb


def apply_points(points, u, nb):
    """A u for per-node stencils (N, 27, 9) and neighbour table nb."""
    N = nb.shape[0]
    pts = points.reshape(N, 27, 3, 3)
    return np.einsum("pbrc,pbc->pr", pts, u.reshape(-1, 3)[nb])


def coeff_grad(mu, lam, spacing, periodic, w, u, dt=1.0):
    """(-w^T dA/dmu_q u, -w^T dA/dlam_q u) for every node q, by probing."""
    o, n, m = mu.shape
    N = m * n * o
    xp, yp, zp = periodic
    per_np = (zp, yp, xp)
    dx, dy, dz = spacing
    nb = neighbours((m, n, o), periodic)
    k, j, i = np.meshgrid(np.arange(o), np.arange(n), np.arange(m), indexing="ij")
    pi, pj, pk = _class_period(m, xp), _class_period(n, yp), _class_period(o, zp)
    cls = (i % pi) + pi * ((j % pj) + pj * (k % pk))
    zero = np.zeros_like(mu)
    out = []
    for which in ("mu", "lam"):
        grad = np.zeros((o, n, m))
        for c in range(pi * pj * pk):
            e = (cls == c).astype(np.float64)
            if not e.any():
                continue
            pts = P.elastic_stencil_points(e if which == "mu" else zero, e if which == "lam" else zero,
                                           dx, dy, dz, periodic, dt=dt)
            Au = apply_points(pts, u, nb)
            r = -(w.reshape(-1, 3) * Au).sum(axis=1).reshape(o, n, m)
            # a node's coefficients are used by its own row and its 6 face neighbours' rows
            s = r.copy()
            for ax in range(3):
                for d in (-1, 1):
                    sh = P._shift(r, d, ax, per_np[ax])
                    s += np.nan_to_num(sh, nan=0.0)
            grad[e.astype(bool)] = s[e.astype(bool)]
        out.append(grad.reshape(N))
    return out[0], out[1]


def gradients(mu, lam, spacing, periodic, b, loss_grad, dt=1.0):
    """u, w and (dL/db, dL/dmu, dL/dlam) of L(u) with dL/du = loss_grad(u)."""
    o, n, m = mu.shape
    pts = P.elastic_stencil_points(mu, lam, *spacing, periodic, dt=dt)
    lu = spla.splu(assemble(pts, (m, n, o), periodic).tocsc(), permc_spec="NATURAL")
    u = lu.solve(np.ascontiguousarray(b, dtype=np.float64).reshape(-1)).reshape(-1, 3)
    g = loss_grad(u)
    w = lu.solve(np.ascontiguousarray(g, dtype=np.float64).reshape(-1), trans="T").reshape(-1, 3)
    dmu, dlam = coeff_grad(mu, lam, spacing, periodic, w, u, dt=dt)
    return u, w, (w, dmu, dlam)
