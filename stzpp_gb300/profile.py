"""Launch one solver kernel on the benchmark workload, for timing and ncu.

    python -m stzpp_gb300.profile --kernel gs --level 0 --precision mixed --reps 20

sets up the 256x256x257 projection problem (the benchmark workload, or
--dims), then launches the chosen kernel 3 + reps times through
stz_mg_time_kernel and prints its time per launch and achieved bandwidth
("sweep" is two whole 8-colour smoother sweeps, several launches).
With --reps 1 the kernel of interest is the 4th launch of its name after
setup, which makes ``ncu -k regex:<name> -s 3 -c 1`` capture exactly it.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import mg as _mg
from . import problems
from .mg import Multigrid, elastic_stencil

KERNELS = {"gs": _mg.K_GS_COLOUR, "sweep": _mg.K_GS_SWEEP, "residual": _mg.K_RESIDUAL,
           "restrict": _mg.K_RESTRICT, "interp": _mg.K_INTERP, "residual64": _mg.K_RESIDUAL64}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", default="256x256x257")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--kernel", default="gs", choices=sorted(KERNELS))
    ap.add_argument("--level", type=int, default=0)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--operator", default="const", choices=["const", "lame"])
    ap.add_argument("--max-coarse", type=int, default=1024)
    ap.add_argument("--setup", action="store_true",
                    help="time the set-up after an operator change (stencil upload + RAT + bottom inverse) instead")
    args = ap.parse_args()
    dims = tuple(int(v) for v in args.dims.split("x"))
    per = (True, True, False)
    h = problems.grid_spacing(dims, per)
    with Multigrid(dims, per, precision=args.precision, max_coarse=args.max_coarse) as m:
        if args.operator == "const":
            m.setup_matrices(*elastic_stencil(1.0, 2.0, *h))
        else:
            mu = problems.lognormal_mu(1, dims).reshape(-1)
            m.setup_matrices(mu=mu, lam=2 * mu, spacing=h)
        if args.setup:
            import time
            st, fix = elastic_stencil(1.0, 2.0, *h)
            times = []
            for rep in range(max(2, args.reps)):
                t0 = time.perf_counter()
                m.setup_matrices(stencil=st * (1.0 + 1e-3 * rep), fix=fix * (1.0 + 1e-3 * rep))
                times.append((time.perf_counter() - t0) * 1e3)
            print(f"setup {args.precision} {args.dims} max_coarse {args.max_coarse} ({m.nlevels} levels): "
                  f"{min(times[1:]):.1f} ms best, {sorted(times[1:])[len(times[1:]) // 2]:.1f} ms median")
            return
        m.set_rhs_divergence(problems.random_strain(0, dims, per), h)
        m.set_x(np.zeros(3 * m.npts))
        ms, work = m.time_kernel(KERNELS[args.kernel], args.level, reps=args.reps)
    unit = "FP64 TFLOP/s" if args.kernel == "residual64" else "GB/s"
    rate = work / (ms * 1e-3) / (1e12 if args.kernel == "residual64" else 1e9)
    print(f"{args.kernel} level {args.level} {args.precision} {args.dims}: {ms * 1e3:.1f} us/launch, "
          f"{rate:.1f} {unit} (algorithmic)")


if __name__ == "__main__":
    main()
