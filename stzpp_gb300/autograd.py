"""Differentiable projection solve on the GPU.

``ProjectionSolver(dims, periodic, spacing)(b, mu, lam)`` returns
u = A(mu, lam)^{-1} b, where A is the variable-coefficient elasticity operator
-dt div(mu (grad u + grad u^T) + lam (div u) I) of the solver's Lame path
(stz_mg_set_coeffs_lame), and is differentiable in b, mu and lam through
:class:`ProjectionSolve`, a ``torch.autograd.Function`` whose backward is the
hand-written adjoint of the C-ABI:

* ``stz_mg_adjoint_solve``: w = A^{-T} dL/du (the multigrid solve of the
  interior block, which is symmetric, plus a node-wise Dirichlet update);
* ``stz_mg_coeff_grad``: dL/dmu, dL/dlam = -w^T (dA/dmu, dA/dlam) u per node.

There is no counterpart in the reference (its solver is not differentiated);
the forward pass is the reference's projection solve (shear_sim_3d.cpp:
567-582).  ``sequence_loss`` chains solves as a simulation loop does and
checkpoints every few solves (``torch.utils.checkpoint``), so a backward pass
through many solves keeps only the segment boundaries.

Tensors are float64 CUDA tensors: b and u of shape (npts, 3), mu and lam of
shape (npts,), natural node order (x fastest).
"""
from __future__ import annotations

import torch

from .mg import Multigrid


class ProjectionSolver:
    """One GPU multigrid handle with the Lame operator, reused across solves.

    ``precision`` "mixed" (FP32 V-cycles inside FP64 defect correction) or
    "fp64"; ``tol`` is the relative residual both the forward and the adjoint
    solves reach.  Coefficients are uploaded (and the hierarchy rebuilt) only
    when a different mu / lam tensor, or a modified one, is passed.
    """

    def __init__(self, dims, periodic=(True, True, False), spacing=None, dt=1.0, precision="mixed", tol=1e-10,
                 max_cycles=200, device=0, **multigrid_kw):
        self.dims = tuple(int(v) for v in dims)
        self.periodic = tuple(bool(p) for p in periodic)
        if spacing is None:
            m, n, o = self.dims
            cells = [m if self.periodic[0] else m - 1, n if self.periodic[1] else n - 1,
                     o if self.periodic[2] else o - 1]
            spacing = tuple(1.0 / c for c in cells)
        self.spacing = tuple(float(h) for h in spacing)
        self.dt = float(dt)
        self.tol = float(tol)
        self.max_cycles = int(max_cycles)
        self.device = torch.device("cuda", device)
        # the handle works on the stream torch is using, so device-side copies
        # in and out are ordered with the caller's kernels
        multigrid_kw.setdefault("stream", torch.cuda.current_stream(self.device).cuda_stream)
        self.mg = Multigrid(self.dims, self.periodic, precision=precision, device=device, **multigrid_kw)
        self._key = None
        self.stats = {"forward_cycles": 0, "adjoint_cycles": 0, "setups": 0}

    @property
    def npts(self):
        m, n, o = self.dims
        return m * n * o

    def close(self):
        self.mg.close()

    @staticmethod
    def _tag(t):
        return (t.data_ptr(), tuple(t.shape), tuple(t.stride()), t._version)

    def set_coefficients(self, mu, lam):
        # The cached tensors are held, so their memory cannot be freed and
        # handed to another tensor: a tensor with the same address, layout and
        # version counter is then a view of the same, unmodified data (the
        # saved-tensor copies autograd and checkpointing hand back are such
        # views).
        if self._key is not None:
            _, tm, _, tl = self._key
            if self._tag(mu) == tm and self._tag(lam) == tl:
                return
        mu_in, lam_in = mu.detach().contiguous(), lam.detach().contiguous()
        torch.cuda.current_stream(self.device).synchronize()
        self.mg.setup_matrices(mu=mu_in, lam=lam_in, spacing=self.spacing, dt=self.dt)
        self._key = (mu, self._tag(mu), lam, self._tag(lam))
        self.stats["setups"] += 1

    def __call__(self, b, mu, lam, x0=None):
        return ProjectionSolve.apply(b, mu, lam, self, x0)

    def rhs_divergence(self, eps):
        """Node divergence of a cell tensor field (6 components per cell, a
        float64 CUDA tensor), assembled on the device by the solver's kernel
        (the r_field of shear_sim_3d); returns a new (npts, 3) tensor.  Uses
        the handle's right-hand side as scratch."""
        eps_in = eps.detach().contiguous()
        torch.cuda.current_stream(self.device).synchronize()
        self.mg.set_rhs_divergence(eps_in, self.spacing)
        out = torch.empty((self.npts, 3), dtype=torch.float64, device=self.device)
        self.mg.get_rhs(out)
        return out


def _check_field(t, shape, name):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64):
        raise TypeError(f"{name} must be a float64 CUDA tensor")
    if tuple(t.shape) != shape:
        raise ValueError(f"{name} must have shape {shape}, got {tuple(t.shape)}")


class ProjectionSolve(torch.autograd.Function):
    """u = A(mu, lam)^{-1} b with the adjoint as backward."""

    @staticmethod
    def forward(ctx, b, mu, lam, solver, x0=None):
        N = solver.npts
        _check_field(b, (N, 3), "b")
        _check_field(mu, (N,), "mu")
        _check_field(lam, (N,), "lam")
        solver.set_coefficients(mu, lam)
        mg = solver.mg
        # Inputs are made on torch's stream and read on the handle's: every
        # tensor the handle reads exists before the synchronize, and each
        # call below returns only after the handle's stream has read it.
        b_in = b.detach().contiguous()
        x_in = torch.zeros_like(b) if x0 is None else x0.detach().contiguous()
        torch.cuda.current_stream(solver.device).synchronize()
        mg.set_rhs(b_in)
        mg.set_x(x_in)
        cycles, _ = mg.solve(solver.tol, solver.max_cycles)
        solver.stats["forward_cycles"] += cycles
        u = torch.empty_like(b)
        mg.get_x(u)
        ctx.solver = solver
        ctx.save_for_backward(u, mu, lam)
        return u

    @staticmethod
    def backward(ctx, gu):
        u, mu, lam = ctx.saved_tensors
        solver = ctx.solver
        solver.set_coefficients(mu, lam)
        g_in = gu.contiguous()
        torch.cuda.current_stream(solver.device).synchronize()
        w, cycles, _ = solver.mg.adjoint_solve(g_in, tol=solver.tol, max_cycles=solver.max_cycles)
        solver.stats["adjoint_cycles"] += cycles
        dmu = dlam = None
        if ctx.needs_input_grad[1] or ctx.needs_input_grad[2]:
            dmu, dlam = solver.mg.coeff_grad(w, u)
        return (w if ctx.needs_input_grad[0] else None, dmu if ctx.needs_input_grad[1] else None,
                dlam if ctx.needs_input_grad[2] else None, None, None)


def sequence_loss(solver, b0, increments, mu, lam, loss_fn, checkpoint_every=10, warm_start=True):
    """Sum over t of loss_fn(t, u_t) for the chain of solves
    A u_t = b_t, b_t = b_{t-1} + increments[t-1] (t = 1..T), b_0 given, each
    solve warm-started from u_{t-1} (the start guess carries no gradient).
    ``increments`` is a sequence of (npts, 3) tensors, or a pair (T, f) with
    f(t) returning increment t (0-based) -- regenerated, not stored, when a
    checkpointed segment is recomputed; f must be deterministic.

    Solves are grouped into segments of ``checkpoint_every``; each segment
    runs under ``torch.utils.checkpoint`` (non-reentrant), so the backward
    pass recomputes a segment's solves instead of storing their solutions.
    ``checkpoint_every`` <= 0 stores everything."""
    from torch.utils.checkpoint import checkpoint

    if isinstance(increments, tuple) and len(increments) == 2 and callable(increments[1]):
        T, inc = increments
    else:
        T, inc = len(increments), increments.__getitem__
    total = torch.zeros((), dtype=torch.float64, device=b0.device)
    b = b0
    x0 = None

    def segment(b_in, mu_, lam_, x_start, t0, t1):
        bb, xx = b_in, x_start
        part = torch.zeros((), dtype=torch.float64, device=b_in.device)
        for t in range(t0, t1):
            bb = bb + inc(t)
            u = solver(bb, mu_, lam_, xx if warm_start else None)
            part = part + loss_fn(t + 1, u)
            xx = u.detach()
        return part, bb, xx

    step = checkpoint_every if checkpoint_every > 0 else T
    for t0 in range(0, T, step):
        t1 = min(T, t0 + step)
        if checkpoint_every > 0:
            part, b, x0 = checkpoint(segment, b, mu, lam, x0, t0, t1, use_reentrant=False)
        else:
            part, b, x0 = segment(b, mu, lam, x0, t0, t1)
        total = total + part
    return total
