"""Seeded synthetic inputs of the benchmark workloads (host side).

The benchmark problems are stzpp's quasi-static projection: periodic x,y,
Dirichlet z plates, the elasticity operator with mu = 1, lambda = 2 (or a
lognormal mu field with lambda = 2 mu), and a right-hand side that is the
node divergence of a random symmetric cell tensor field.  Only the random
draws happen here (numpy PCG64); the right-hand side itself is assembled on
the GPU (Multigrid.set_rhs_divergence).
"""
from __future__ import annotations

import numpy as np


def grid_spacing(dims, periodic, h=None):
    """1/N per dimension (N cells: nodes for a periodic dimension, nodes-1
    otherwise), or a uniform spacing h."""
    if h is not None:
        return (h, h, h)
    return tuple(1.0 / (d if p else d - 1) for d, p in zip(dims, periodic))


def cell_counts(dims, periodic):
    return tuple(d if p else d - 1 for d, p in zip(dims, periodic))


def random_strain(seed, dims, periodic, std=1e-3):
    """Cell tensor field, shape (cells_z, cells_y, cells_x, 6): i.i.d. N(0, std)
    components (s11, s12, s13, s22, s23, s33)."""
    mc, nc, oc = cell_counts(dims, periodic)
    rng = np.random.default_rng(seed)
    return rng.standard_normal(size=(oc, nc, mc, 6)) * std


def lognormal_mu(seed, dims, sigma=0.3):
    """Per-node mu = exp(sigma Z), Z ~ N(0,1): median 1.  Shape (o, n, m)."""
    m, n, o = dims
    rng = np.random.default_rng(seed)
    return np.exp(sigma * rng.standard_normal(size=(o, n, m)))
