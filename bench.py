#!/usr/bin/env python3
"""Benchmark: stzpp's quasi-static projection solve on one GB300.

Workload (the 257^3 problem): 256 x 256 x 257 nodes -- periodic x and y with
256 cells, Dirichlet plates in z with 256 cells -- dx = 1/256, the elasticity
operator with mu = 1, lambda = 2 (the shared 27-block stencil of
shear_sim_3d::set_up_stencil_base), right-hand side = node divergence of a
random symmetric cell tensor field with i.i.d. N(0, 1e-3) entries (seed 0),
zero initial guess, V-cycles until |b - Ax| / |b| <= 1e-10.

One step = one solve.  `value` is ms per solve in mixed precision (FP32
V-cycles inside FP64 defect correction) with every input resident in HBM;
`e2e` is the same solve through the C-ABI from pinned host buffers (RHS
host->device, solution device->host inside the timed region).  The plain FP64
GPU solve is timed beside it.  Fine-level vectors are 404 MB each (larger
than the 129 MB L2), so no L2 flush is needed between steps.

--impl reference times the reference algorithm (its C restatement in
oracle/, pinned to the compiled reference by the tests) on all host cores at
the same size: a full solve, then timed V-cycles at full size, and prints the
same metric.  The default run also times one full reference solve as its
cpu_baseline and compares the GPU solutions with the reference's.

Runs as N independent replicas under torchrun (--gpus N): the solve is not
sharded in this build.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/solve to rel. residual 1e-10 at 257³, mixed vs FP64 on GPU; smoother % HBM"
DIMS = (256, 256, 257)
PERIODIC = (True, True, False)
TOL = 1e-10
WORKLOAD = ("quasi-static projection solve, 256x256x257 nodes (257^3 problem: periodic x,y, Dirichlet z), "
            "mu=1, lambda=2, dx=1/256, RHS = divergence of N(0,1e-3) cell strain (seed 0), x0 = 0, "
            "to relative residual 1e-10")
# Cycle of the GPU solves: two sweeps down, four up on every level.  Measured
# at 256x256x257 on a GB300 with the band sweeps (mixed ms per solve, cycles):
# V(2,4) 24.3 (10), V(2,3) 25.8 (11), V(2,2) 26.6 (14), V(3,3) 30.7 (10),
# V(4,4) 34.2 (10): pairs of sweeps run as band sweeps, an odd one as eight
# colour launches, so even counts pay off.  With the colour launches alone
# (earlier kernels) V(2,3) was best: 41.8 ms against V(2,2) 44.2, V(3,3) 43.5,
# and the reference's growing schedule (v + i sweeps on level i) V(2,2) 46.0.
V_DOWN, V_UP = 2, 4


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile(name):
    """DRAM bytes per launch of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(name)
    except Exception:
        return None


class Clocks:
    """nvidia-smi clock / throttle sampling around a timed region: the sampler
    starts before the warm-up (nvidia-smi takes a moment to come up), samples
    every 50 ms, and only the samples stamped between mark() and stop() count
    (all samples if the stamps cannot be read)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_index, interval_ms=50):
        self.gpu = gpu_index
        self.interval_ms = interval_ms
        self.proc = None
        self.t0 = None

    def start(self):
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def mark(self):
        """The timed region starts now."""
        self.t0 = datetime.datetime.now()

    def stop(self):
        t1 = datetime.datetime.now()
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.flush()
        lines = [l for l in open(self.out.name) if l.strip()]
        os.unlink(self.out.name)
        return self.summarise(lines, self.t0, t1)

    @classmethod
    def summarise(cls, lines, t0, t1):
        """Median SM clock, max clock and active throttle reasons of the
        sample lines stamped within [t0, t1] (of every line when no stamp in
        the window can be read)."""
        rows = []
        for l in lines:
            r = [v.strip() for v in l.split(",")]
            if len(r) < 10:
                continue
            try:
                sm, mx = float(r[2]), float(r[3])
            except ValueError:
                continue
            try:
                ts = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                ts = None
            rows.append((ts, sm, mx, r[6:10]))
        window = "timed region"
        inside = [x for x in rows if t0 is not None and x[0] is not None and t0 <= x[0] <= t1]
        if not inside:
            inside, window = rows, "sampler lifetime (warm-up and timed region)"
        if not inside:
            return None
        reasons = set()
        for _, _, _, flags in inside:
            for n, v in zip(cls.REASONS, flags):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(x[1] for x in inside), "sm_max_mhz": max(x[2] for x in inside),
                "reasons": sorted(reasons), "samples": len(inside), "window": window}


def reduce_max(value, dist, device):
    """Max of a per-rank scalar over all ranks (the slowest replica sets the
    job's time); returns the value itself on a single process."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_ms_per_solve(max_ms_per_step, world):
    """Whole-job ms per solve of `world` replicas that each ran one solve per
    step in max_ms_per_step (time-like metric: total time / total solves)."""
    return max_ms_per_step / world


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


REF_SOLVER = ("the reference algorithm, restated in C (oracle/): multigrid<vec3,mat3> with the shared stencil, "
              "lexicographic block GS V(2+i,2+i), RAT coarse operators, coarsest level <= 1024 nodes with 24 GS "
              "sweeps; on T host threads as T z-slab sub-domains with ghosts refreshed once per sweep (the "
              "reference's MPI decomposition along z)")
# tolerance of the solutions compared between the GPU and the reference: both
# converged well below the timed 1e-10, so their difference measures the
# solvers, not the stopping points
PARITY_TOL = 1e-12


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def reference_rhs():
    """b of the headline workload in natural order, assembled on the host by
    the oracle (the GPU arm assembles the same values on the device)."""
    from oracle import problem as P
    from stzpp_gb300 import problems
    m, n, o = DIMS
    h = P.grid_spacing(m, n, o, PERIODIC)
    return P.rhs_divergence(problems.random_strain(0, DIMS, PERIODIC), m, n, o, PERIODIC, *h)


def reference_solver(b, threads):
    """The reference algorithm at 256x256x257 on `threads` host threads:
    set-up, then one solve from x = 0 to |b - Ax|/|b| <= 1e-10 timed as the
    reference's loop runs it (V-cycle, then the FP64 residual norm), then on to
    1e-12 (untimed) for the solution comparisons.  Returns (handle, record,
    solution at 1e-12)."""
    from oracle import port, problem as P
    if not port.available():
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    used = port.set_threads(threads)
    m, n, o = DIMS
    st, fix = P.elastic_stencil_const(1.0, 2.0, *P.grid_spacing(m, n, o, PERIODIC))
    t0 = time.perf_counter()
    M = port.PortMultigrid(DIMS, PERIODIC, stencil=st, fix=fix, max_coarse=1024)
    setup_s = time.perf_counter() - t0
    M.set_field(0, "r", b)
    M.set_field(0, "x", np.zeros_like(b))
    t0 = time.perf_counter()
    cycles, hist = M.solve(TOL, 200, bottom="gs", smoother="lex")
    solve_s = time.perf_counter() - t0
    c2, hist2 = M.solve(PARITY_TOL, 200, bottom="gs", smoother="lex")
    rec = {"threads": used, "setup_s": setup_s, "solve_ms": solve_s * 1e3, "cycles": int(cycles),
           "relres": float(hist[-1]) if len(hist) else None, "parity_cycles": int(cycles + c2),
           "parity_relres": float(hist2[-1]) if len(hist2) else None}
    return M, rec, M.get_field(0, "x")


def rel_err(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_reference(args, world, rank):
    """The reference arm: the reference algorithm on all host threads at the
    headline size.  One full solve to 1e-10 first (its cycle count and wall
    time), then W untimed and K timed steps, each step one V-cycle plus the
    residual norm (the body of the reference's solve loop) at full size;
    ms per solve = ms per step x the cycles of the full solve.  Other ranks
    exit without work."""
    if rank != 0:
        return
    threads = host_threads()
    b = reference_rhs()
    M, rec, _ = reference_solver(b, threads)
    for _ in range(args.warmup):
        M.v_cycle(bottom="gs", smoother="lex")
        M.residual_sq(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        M.v_cycle(bottom="gs", smoother="lex")
        M.residual_sq(0)
    ms_step = (time.perf_counter() - t0) * 1e3 / args.steps
    value = ms_step * rec["cycles"]
    sample = (f"{args.steps} timed V-cycles + residual norms at 256x256x257 ({ms_step:.0f} ms each) x the "
              f"{rec['cycles']} cycles the full solve to 1e-10 took; that full solve, timed whole: "
              f"{rec['solve_ms']:.0f} ms")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(args, world), "reference_solver": REF_SOLVER,
            "full_solve": rec,
            "cpu_baseline": {"value": value, "unit": "ms", "cores": rec["threads"], "kind": "port",
                             "sample": sample, "host_cores_available": os.cpu_count()},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def headline_config(args, world):
    return {"workload": WORKLOAD, "dims": list(DIMS),
            "precision": ("mixed: FP32 V-cycles; top residual of each correction step in double-float arithmetic "
                          "(FP32 pairs, ~2^-47) from the FP64 x and b; FP64 update and bottom"),
            "cycle": (f"V({args.v_down},{args.v_up}) on every level, 8-colour block GS, RAT coarse operators "
                      f"(plane-invariant storage), FP64 direct solve of the coarsest level "
                      f"(<= {args.max_coarse} nodes)"),
            "replicas": world, "l2": "inputs larger than L2 (fine vectors 404 MB each); no flush needed"}


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import stzpp_gb300 as sg
    from stzpp_gb300 import problems
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if dist.is_nccl_available() else "gloo")
    dims, per = DIMS, PERIODIC
    npts = dims[0] * dims[1] * dims[2]
    # the end-to-end leg's pinned host buffers, allocated before the device
    # memory of the handles
    b_host = torch.empty(3 * npts, dtype=torch.float64, pin_memory=True)
    x_host = torch.empty(3 * npts, dtype=torch.float64, pin_memory=True)
    spacing = problems.grid_spacing(dims, per)
    stencil, fix = sg.elastic_stencil(1.0, 2.0, *spacing)
    eps = problems.random_strain(0, dims, per)
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(v):
        return reduce_max(v, dist, "cuda" if dist is None or dist.get_backend() == "nccl" else "cpu")

    # ---------------------------------------------------------- mixed solve
    mg = sg.Multigrid(dims, per, precision="mixed", v_down=args.v_down, v_up=args.v_up,
                      sweep_growth=bool(args.sweep_growth), max_coarse=args.max_coarse, device=local,
                      stream=stream.cuda_stream)
    t0 = time.perf_counter()
    mg.setup_matrices(stencil=stencil, fix=fix)
    torch.cuda.synchronize()
    setup_ms = (time.perf_counter() - t0) * 1e3
    mg.set_rhs_divergence(eps, spacing)
    b_dev = torch.empty(3 * npts, dtype=torch.float64, device="cuda")
    mg.get_rhs(b_dev)
    zero = torch.zeros_like(b_dev)

    def step(M):
        M.set_x(zero)
        return M.solve(TOL, 200)

    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        step(mg)
    barrier()
    clocks.mark()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    cycles = 0
    for _ in range(args.steps):
        cycles, rel = step(mg)
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms_mixed = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    vcyc, nres, launches = mg.solve_stats()
    x_mixed = torch.empty_like(b_dev)
    mg.get_x(x_mixed)
    rn64, bn64 = mg.residual_norm()   # the FP64 residual of the mixed result

    # ------------------------------------------------- end to end (C-ABI)
    b_host.copy_(b_dev)
    e2e_steps = max(2, args.steps // 2)

    copy_s = [0.0, 0.0]

    def e2e_step():
        t = time.perf_counter()
        mg.set_rhs(b_host)          # host -> device
        copy_s[0] += time.perf_counter() - t
        mg.set_x(zero)
        mg.solve(TOL, 200)
        t = time.perf_counter()
        mg.get_x(x_host)            # device -> host
        copy_s[1] += time.perf_counter() - t

    e2e_step()   # untimed: the first copies into freshly pinned pages map them
    copy_s[0] = copy_s[1] = 0.0
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    barrier()
    ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps)

    # ------------------------------------------- the simulation drivers' loop
    # shear_sim_3d::projection_step (shear_sim_3d.cpp:554-599): v_cycle(); err
    # = l2_error_all() (sum of |r|^4) until err <= (1e3 eps A_c11)^2, then two
    # more cycles; through the same C-ABI calls the C++ adapter makes
    l2_tol = (np.finfo(float).eps * abs(np.asarray(stencil).reshape(27, 9)[13, 0]) * 1e3) ** 2

    def driver_solve():
        mg.set_x(zero)
        n, err = 0, float("inf")
        while err > l2_tol and n < 200:
            mg.v_cycle()
            n += 1
            err = mg.l2_error_all()
        mg.v_cycle()
        mg.v_cycle()
        return n + 2

    driver_solve()   # warm-up
    barrier()
    e0.record(stream)
    drv_cycles = driver_solve()
    e1.record(stream)
    barrier()
    ms_driver = max_over_ranks(e0.elapsed_time(e1))
    drv_rn, drv_bn = mg.residual_norm()
    driver_loop = {"ms_per_solve": ms_driver, "v_cycles": drv_cycles, "relres_fp64": drv_rn / drv_bn,
                   "stop": "sum |r|^4 <= (1e3 eps A_c11)^2, then two more cycles",
                   "note": "each mixed v_cycle is one defect-correction step of one FP32 cycle; l2_error_all's "
                           "residual is reused as the next step's right-hand side"}

    # -------------------------------------------------- kernel roofline
    hbm, hbm_kind = peaks()
    kern = {}
    for name, kid, lvl in (("gs_colour_l0", sg.mg.K_GS_COLOUR, 0), ("gs_colour_l1", sg.mg.K_GS_COLOUR, 1),
                           ("gs_sweep_l0", sg.mg.K_GS_SWEEP, 0),
                           ("residual_l0_fp32", sg.mg.K_RESIDUAL, 0), ("restrict_l1", sg.mg.K_RESTRICT, 1),
                           ("interp_l1", sg.mg.K_INTERP, 1), ("residual_top", sg.mg.K_RESIDUAL64, 0)):
        ms, work = mg.time_kernel(kid, lvl, reps=10 if kid == sg.mg.K_GS_SWEEP else 20)
        kern[name] = (ms, work)
    # the fine-level smoother as the solve runs it, timed over two whole
    # sweeps: the band sweep (two launches per sweep: the four colours of every
    # even, then every odd plane) or the eight colour launches; per launch
    kind, lps = mg.sweep_kind(0)
    sw_ms, sw_bytes = kern["gs_sweep_l0"]
    gs_ms, gs_bytes = sw_ms / (2 * lps), sw_bytes / (2 * lps)
    achieved = gs_bytes / (gs_ms * 1e-3) / 1e9
    # sweeps per cycle on the fine level: whole pairs run as band sweeps, an
    # odd last one as eight colour launches
    sweeps = args.v_down + args.v_up
    paired = (args.v_down // 2 + args.v_up // 2) * 2 if kind == "band" else sweeps
    gs_launches = paired * lps * vcyc
    r64_ms, r64_flops = kern["residual_top"]
    if kind == "band":
        kname, tkey = ("gs_band_kernel<float,128> (fine-level band sweep: one launch = the four colours of every "
                       "even or every odd plane, bands of 8 rows staged by TMA; the average over two whole sweeps)",
                       "gs_band_kernel<float>")
        tnote = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch (profiles/gs_band_fine_256x256x257.md)")
    else:
        kname, tkey = ("gs_const_kernel<float> (fine-level 8-colour GS: one colour pass, the average over two "
                       "whole sweeps)", "gs_const_kernel<float>")
        tnote = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of colour 0 repeated alone "
                 "(profiles/gs_const_fine_256x256x257.md)")
    roofline = {"kernel": kname,
                "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "peak_kind": f"{hbm_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)" if hbm_kind == "measured" else hbm_kind,
                "traffic": traffic_from_profile(tkey), "traffic_note": tnote,
                "algorithmic_bytes_per_launch": gs_bytes, "ms_per_launch": gs_ms,
                "launches_per_solve": gs_launches,
                "share_of_solve_est": gs_launches * gs_ms / ms_mixed}
    smoother = {name: {"ms_per_launch": v[0], "GB/s": v[1] / (v[0] * 1e-3) / 1e9,
                       "frac_hbm": v[1] / (v[0] * 1e-3) / 1e9 / hbm}
                for name, v in kern.items() if name != "residual_top"}
    # the correction steps' top residual: split of the FP64 x into float pairs
    # + double-float b - A x (exact products, compensated sums) + block sums;
    # rate in the flops of the FP64 formulation (2 x 51 per node)
    smoother["residual_top"] = {"ms_per_launch": r64_ms, "arithmetic": "double-float (FP32 pairs) from FP64 x, b",
                                "FP64-equivalent TFLOP/s": r64_flops / (r64_ms * 1e-3) / 1e12,
                                "launches_per_solve": nres}
    mg.close()

    # ------------------------------------------------------ FP64 solve
    mg64 = sg.Multigrid(dims, per, precision="fp64", v_down=V_DOWN, v_up=V_UP, sweep_growth=False,
                        max_coarse=args.max_coarse, device=local, stream=stream.cuda_stream)
    mg64.setup_matrices(stencil=stencil, fix=fix)
    mg64.set_rhs(b_dev)
    steps64 = max(2, args.steps // 2)
    for _ in range(min(args.warmup, 2)):
        step(mg64)
    barrier()
    e0.record(stream)
    for _ in range(steps64):
        cyc64, rel64 = step(mg64)
    e1.record(stream)
    barrier()
    ms_fp64 = max_over_ranks(e0.elapsed_time(e1) / steps64)
    x64 = torch.empty_like(b_dev)
    mg64.get_x(x64)
    mg64.close()
    err = float(torch.linalg.norm(x_mixed - x64) / torch.linalg.norm(x64))

    # the reference algorithm on the host cores, same workload and inputs:
    # one full solve (the CPU baseline), and its solution to 1e-12 for parity
    # with the GPU's FP64 solution to 1e-12 (config 2: <= 1e-9 relative L2)
    cpu, parity = None, None
    if rank == 0 and world == 1:
        b_nat = b_dev.cpu().numpy().reshape(-1, 3)
        M, rec, x_ref = reference_solver(b_nat, host_threads())
        del M
        cpu = {"value": rec["solve_ms"], "unit": "ms", "cores": rec["threads"], "kind": "port",
               "sample": (f"one full solve at 256x256x257 to 1e-10 from x = 0 ({rec['cycles']} V-cycles, "
                          f"relres {rec['relres']:.2e}), {REF_SOLVER}"),
               "host_cores_available": os.cpu_count(), "setup_s": rec["setup_s"]}
        mgp = sg.Multigrid(dims, per, precision="fp64", v_down=V_DOWN, v_up=V_UP, sweep_growth=False,
                           max_coarse=args.max_coarse, device=local, stream=stream.cuda_stream)
        mgp.setup_matrices(stencil=stencil, fix=fix)
        mgp.set_rhs(b_dev)
        mgp.set_x(zero)
        cyc_t, rel_t = mgp.solve(PARITY_TOL, 300)
        x_tight = mgp.get_x()
        mgp.close()
        parity = {"tolerance": PARITY_TOL, "reference_relres": rec["parity_relres"], "gpu_fp64_relres": rel_t,
                  "gpu_fp64_vs_reference": rel_err(x_tight, x_ref),
                  "timed_fp64_1e-10_vs_reference": rel_err(x64.cpu().numpy(), x_ref),
                  "timed_mixed_1e-10_vs_reference": rel_err(x_mixed.cpu().numpy(), x_ref),
                  "bound": 1e-9}
    if rank == 0:
        value = job_ms_per_solve(ms_mixed, world)
        line = {
            "metric": METRIC, "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": headline_config(args, world),
            "cycles": cycles, "relres": rel, "relres_fp64": rn64 / bn64,
            "relres_note": ("relres: the mixed solver's stopping test (double-float residual); relres_fp64: "
                            "|b - A x| / |b| of the same x in FP64"), "setup_ms": setup_ms,
            "fp64": {"ms_per_solve": ms_fp64, "cycles": cyc64, "relres": rel64},
            "speedup_vs_fp64": ms_fp64 / ms_mixed, "solution_rel_err_vs_fp64": err,
            "roofline": roofline, "kernels": smoother, "driver_loop": driver_loop,
            "e2e": {"value": job_ms_per_solve(ms_e2e, world), "unit": "ms", "h2d_bytes_per_step": 3 * npts * 8,
                    "d2h_bytes_per_step": 3 * npts * 8,
                    "h2d_ms_per_step": copy_s[0] * 1e3 / e2e_steps, "d2h_ms_per_step": copy_s[1] * 1e3 / e2e_steps},
            "gpu_launches": int(launches * args.steps),
            "clocks": clk,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
            line["solution_rel_err_vs_reference"] = parity
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------------ config 3
C3_DIMS = (512, 512, 257)
C3_H = 1.0 / 256   # the grid spacing of the 257^3 problem on a 2 x 2 x 1 box


def run_config3(args, local):
    """512x512x257, lognormal mu (median 1, sigma 0.3, seed 1), lambda = 2 mu:
    mixed vs FP64 GPU solve to 1e-10 and the mixed solution's error against
    the FP64 one."""
    import torch
    torch.cuda.set_device(local)
    import stzpp_gb300 as sg
    from stzpp_gb300 import problems
    dims, per, h = C3_DIMS, PERIODIC, (C3_H, C3_H, C3_H)
    npts = dims[0] * dims[1] * dims[2]
    stream = torch.cuda.current_stream()
    mu_d = torch.from_numpy(problems.lognormal_mu(1, dims).reshape(-1)).cuda()
    lam_d = 2 * mu_d
    eps = torch.from_numpy(problems.random_strain(0, dims, per)).cuda()
    res = {}
    x_mixed = None
    for prec in ("mixed", "fp64"):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        t0 = time.perf_counter()
        mg = sg.Multigrid(dims, per, precision=prec, sweep_growth=False, device=local, stream=stream.cuda_stream)
        mg.setup_matrices(mu=mu_d, lam=lam_d, spacing=h)
        torch.cuda.synchronize()
        setup_ms = (time.perf_counter() - t0) * 1e3
        mem = free0 - torch.cuda.mem_get_info()[0]
        mg.set_rhs_divergence(eps, h)
        zero = torch.zeros(3 * npts, dtype=torch.float64, device="cuda")
        steps = max(1, args.steps // (2 if prec == "mixed" else 3))
        for _ in range(max(1, min(args.warmup, 2 if prec == "mixed" else 1))):
            mg.set_x(zero)
            mg.solve(TOL, 300)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            mg.set_x(zero)
            cyc, rel = mg.solve(TOL, 300)
        e1.record(stream)
        torch.cuda.synchronize()
        x = torch.empty(3 * npts, dtype=torch.float64, device="cuda")
        mg.get_x(x)
        res[prec] = {"ms_per_solve": e0.elapsed_time(e1) / steps, "cycles": cyc, "relres": rel,
                     "setup_ms": setup_ms, "device_bytes": int(mem), "levels": mg.nlevels}
        mg.close()
        if prec == "mixed":
            x_mixed = x
        else:
            res["solution_rel_err_mixed_vs_fp64"] = float(torch.linalg.norm(x_mixed - x) / torch.linalg.norm(x))
        del x
    line = {"metric": "ms/solve to rel. residual 1e-10, mixed vs FP64 on GPU (512x512x257, lognormal mu)",
            "value": res["mixed"]["ms_per_solve"], "unit": "ms", "higher_is_better": False,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "512x512x257 nodes, periodic x,y, Dirichlet z, h = 1/256, Lame operator with "
                                   "lognormal mu (median 1, sigma 0.3, seed 1), lambda = 2 mu, RHS = divergence of "
                                   "N(0,1e-3) cell strain (seed 0), x0 = 0, rel. residual 1e-10",
                       "cycle": "V(2,2), 8-colour block GS, RAT (dense coarse levels), FP64 direct bottom"},
            "mixed": res["mixed"], "fp64": res["fp64"],
            "speedup_vs_fp64": res["fp64"]["ms_per_solve"] / res["mixed"]["ms_per_solve"],
            "solution_rel_err_mixed_vs_fp64": res["solution_rel_err_mixed_vs_fp64"]}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ config 5
def run_config5(args, local, T=50, every=10):
    """50 warm-started mixed solves at 256x256x257 with a fixed lognormal mu,
    b_t = b_{t-1} + divergence of an N(0,1e-5) strain-rate field (seeds from
    3), loss sum_t |u_t - u*|^2 (u* ~ N(0,1e-3), seed 2); backward through all
    solves with checkpointing every 10; gradient error against the FP64
    solver (tolerance 1e-12) on the same sequence."""
    import torch
    torch.cuda.set_device(local)
    from stzpp_gb300 import problems
    from stzpp_gb300.autograd import ProjectionSolver, sequence_loss
    dims, per = DIMS, PERIODIC
    npts = dims[0] * dims[1] * dims[2]
    h = problems.grid_spacing(dims, per)
    ncells = dims[0] * dims[1] * (dims[2] - 1)
    mu0 = torch.from_numpy(problems.lognormal_mu(1, dims).reshape(-1)).cuda()
    ustar = torch.from_numpy(np.random.default_rng(2).normal(0.0, 1e-3, size=(npts, 3))).cuda()
    eps0 = torch.from_numpy(problems.random_strain(0, dims, per)).cuda()

    def run(prec, tol, ck, T=T):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        S = ProjectionSolver(dims, per, h, precision=prec, tol=tol, max_cycles=300, sweep_growth=False)
        b0 = S.rhs_divergence(eps0).requires_grad_(True)
        mu = mu0.clone().requires_grad_(True)
        lam = (2 * mu0).clone().requires_grad_(True)
        S.set_coefficients(mu, lam)

        def inc(t):
            g = torch.Generator(device="cuda")
            g.manual_seed(3000 + t)
            return S.rhs_divergence(torch.randn(ncells * 6, generator=g, dtype=torch.float64, device="cuda") * 1e-5)

        torch.cuda.synchronize()
        handle_bytes = free0 - torch.cuda.mem_get_info()[0]
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        t0 = time.perf_counter()
        L = sequence_loss(S, b0, (T, inc), mu, lam, lambda t, u: ((u - ustar) ** 2).sum(), checkpoint_every=ck)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        L.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out = {"forward_ms": (t1 - t0) * 1e3, "backward_ms": (t2 - t1) * 1e3,
               "peak_tensor_bytes": int(torch.cuda.max_memory_allocated() - base),
               "solver_bytes": int(handle_bytes), "setups": S.stats["setups"],
               "forward_cycles": S.stats["forward_cycles"],
               "adjoint_cycles": S.stats["adjoint_cycles"], "loss": float(L.detach())}
        grads = (b0.grad.detach().clone(), mu.grad.detach().clone(), lam.grad.detach().clone())
        S.close()
        return out, grads

    run("mixed", TOL, 2, T=4)   # warm-up: first-use costs of the process stay out of the timings
    mixed, g_mixed = run("mixed", TOL, every)
    stored, _ = run("mixed", TOL, 0)
    fp64, g_64 = run("fp64", 1e-12, every)
    err = [float(torch.linalg.norm(a - r) / torch.linalg.norm(r)) for a, r in zip(g_mixed, g_64)]
    line = {"metric": "50-solve sequence, forward/backward ms with checkpointing (256x256x257, mixed)",
            "value": mixed["forward_ms"] + mixed["backward_ms"], "unit": "ms", "higher_is_better": False,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "50 warm-started solves, 256x256x257, h = 1/256, Lame operator, lognormal mu "
                                   "(sigma 0.3, seed 1), lambda = 2 mu, b_t = b_{t-1} + div(N(0,1e-5) strain rate, "
                                   "seeds 3000+t), loss sum_t |u_t - u*|^2, u* ~ N(0,1e-3) seed 2",
                       "checkpoint_every": every},
            "mixed_checkpointed": mixed, "mixed_stored": stored, "fp64_checkpointed": fp64,
            "gradient_rel_err_vs_fp64": {"b0": err[0], "mu": err[1], "lam": err[2]}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ coefficient change
def run_coeff_change(args, local, steps=12):
    """The trans_sim per-step path: each step uploads a new transformed-frame
    shared stencil (the reference's own stencils of trans_sim_3d for three
    frames, tests/golden/trans_stencils.npz, cycled), rebuilds the hierarchy
    (RAT + bottom inverse), and solves the 256x256x257 projection to 1e-10 in
    mixed precision warm-started from the previous step."""
    import torch
    torch.cuda.set_device(local)
    import stzpp_gb300 as sg
    from stzpp_gb300 import problems
    dims, per = DIMS, PERIODIC
    h = 1.0 / 256
    d = np.load(os.path.join(ROOT, "tests", "golden", "trans_stencils.npz"))
    frames = [(d["stencil"][c].reshape(27, 9) / (h * h), d["fix"][c] / (h * h)) for c in range(len(d["T"]))]
    stream = torch.cuda.current_stream()
    out = {}
    for mc in (1024, 16):
        mg = sg.Multigrid(dims, per, precision="mixed", sweep_growth=False, max_coarse=mc, device=local,
                          stream=stream.cuda_stream)
        mg.setup_matrices(*frames[0])
        mg.set_rhs_divergence(problems.random_strain(0, dims, per), (h, h, h))
        mg.set_x(np.zeros(3 * mg.npts))
        t_set, t_solve, cyc = [], [], []
        for s in range(steps + 2):
            st, fix = frames[s % len(frames)]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mg.setup_matrices(stencil=st, fix=fix)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            c, rel = mg.solve(TOL, 300)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            if s >= 2:
                t_set.append((t1 - t0) * 1e3)
                t_solve.append((t2 - t1) * 1e3)
                cyc.append(c)
        out[f"max_coarse_{mc}"] = {"levels": mg.nlevels, "setup_ms": statistics.median(t_set),
                                   "solve_ms": statistics.median(t_solve), "cycles": cyc,
                                   "step_ms": statistics.median([a + b for a, b in zip(t_set, t_solve)])}
        mg.close()
    line = {"metric": "ms per coefficient-change step (new shared stencil + set-up + solve to 1e-10), 256x256x257 mixed",
            "value": out["max_coarse_16"]["step_ms"], "unit": "ms", "higher_is_better": False, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "256x256x257, h = 1/256, the reference's trans_sim_3d stencils for 3 frames "
                                   "(full non-symmetric 3x3 blocks), cycled; RHS = divergence of N(0,1e-3) strain "
                                   "(seed 0); each solve warm-started from the previous step", "steps": steps},
            **out}
    print(json.dumps(line), flush=True)


# Algorithmic bytes of one advection step per interior cell: read u, v, w,
# the 6 stresses, chi, the previous ad_Dpl and cchi; write the 6 stress
# changes, cchi, sbar and ad_Dpl (21 doubles).
ADV_BYTES_PER_CELL = 21 * 8


def advection_fields(n, seed, device):
    """Seeded fields of an n^3 ghosted grid, made on the device: velocities
    N(0, 1e-3); stress tensors of random direction scaled to a deviatoric
    magnitude sbar ~ U(0.5, 1.15) (in units of the yield stress: about 23 % of
    the cells above it, as in a shear band of a running simulation); chi about
    550 K; previous ad_Dpl U(0, 1e-3); ghosts periodic in x and y, random in z."""
    import torch
    from stzpp_gb300 import advect
    g = advect.NGHOST
    gen = torch.Generator(device=device).manual_seed(seed)
    shape = (n + 2 * g,) * 3
    f = {}
    for k in advect.INPUTS + advect.OUTPUTS:
        t = torch.zeros(shape, dtype=torch.float64, device=device)
        if k in ("u", "v", "w"):
            t.normal_(0, 1e-3, generator=gen)
        elif k.startswith("s") and k != "sbar":
            t.normal_(0, 1.0, generator=gen)
        elif k == "chi":
            t.normal_(550 / 21000, 15 / 21000, generator=gen)
        elif k == "ad_dpl":
            t.uniform_(0, 1e-3, generator=gen)
        f[k] = t
    p = -(f["s11"] + f["s22"] + f["s33"]) / 3
    dev = torch.sqrt(0.5 * ((f["s11"] + p) ** 2 + (f["s22"] + p) ** 2 + (f["s33"] + p) ** 2) +
                     f["s12"] ** 2 + f["s13"] ** 2 + f["s23"] ** 2)
    target = torch.empty(shape, dtype=torch.float64, device=device).uniform_(0.5, 1.15, generator=gen)
    scale = target / dev
    for k in ("s11", "s12", "s13", "s22", "s23", "s33"):
        f[k] *= scale
    for k, t in f.items():
        t[:, :, :g] = t[:, :, n:n + g]
        t[:, :, n + g:] = t[:, :, g:2 * g]
        t[:, :g] = t[:, n:n + g]
        t[:, n + g:] = t[:, g:2 * g]
        f[k] = t.reshape(-1)
    return f


def run_advection(args, local, n=256, dt=200.0):
    """The quasi-static advection step of shear_sim_3d (the part of a
    step_forward_qs before the projection solve) on a 256^3-cell grid at the
    reference driver's quasi-static step (dt = tf / N_tp / qs_steps = 4e5 /
    200 / 10, shear_sim.cpp:58-60): ms per step with the fields resident in
    HBM, and end to end with the inputs copied from pinned host memory and the
    outputs copied back every step."""
    import torch
    torch.cuda.set_device(local)
    sys.path.insert(0, ROOT)
    from oracle import advect as A
    from stzpp_gb300 import advect
    dims = (n, n, n)
    sp = (1.0 / n,) * 3
    prm = A.driver_params(n)
    f = advection_fields(n, 0, f"cuda:{local}")
    work = torch.empty(advect.work_size(*dims), dtype=torch.float64, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    yielded = advect.advection_step(f, dims, sp, prm, dt, work=work)
    plastic = float((f["ad_dpl"].reshape((n + 4,) * 3)[2:-2, 2:-2, 2:-2] > 0).double().mean())
    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        advect.advection_step(f, dims, sp, prm, dt, work=work, wait=False)
    torch.cuda.synchronize()
    clocks.mark()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        advect.advection_step(f, dims, sp, prm, dt, work=work, wait=False)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    # end to end: every step copies the 12 input fields in and the 9 changed ones out
    ins = list(advect.INPUTS) + ["ad_dpl", "cchi"]
    host_in = {k: torch.empty_like(f[k], device="cpu").pin_memory() for k in ins}
    host_out = {k: torch.empty_like(f[k], device="cpu").pin_memory() for k in advect.OUTPUTS}
    for k in ins:
        host_in[k].copy_(f[k])
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        for k in ins:
            f[k].copy_(host_in[k], non_blocking=True)
        advect.advection_step(f, dims, sp, prm, dt, work=work, wait=False)
        for k in advect.OUTPUTS:
            host_out[k].copy_(f[k], non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    npts = advect.grid_points(*dims)
    # CPU baseline: the C restatement on a 48^3 sample of the same fields, scaled by cells
    m = 48
    fs = advection_fields(m, 0, f"cuda:{local}")
    Fs = np.zeros((advect.grid_points(m, m, m), A.NFIELD))
    for k, c in (("u", A.U), ("v", A.V), ("w", A.W), ("s11", A.S11), ("s12", A.S12), ("s13", A.S13),
                 ("s22", A.S22), ("s23", A.S23), ("s33", A.S33), ("chi", A.CHI), ("ad_dpl", A.ADPL)):
        Fs[:, c] = fs[k].cpu().numpy()
    t0 = time.perf_counter()
    A.port_step(Fs, m, m, m, A.driver_params(m), dt)
    cpu_ms = (time.perf_counter() - t0) * 1e3 * (n / m) ** 3
    peak, kind = peaks()
    achieved = ADV_BYTES_PER_CELL * n ** 3 / (ms * 1e-3) / 1e9
    line = {"metric": f"ms per quasi-static advection step (shear_sim_3d::advection_step), {n}^3 cells",
            "value": ms, "unit": "ms", "higher_is_better": False, "dtype": "f64", "data": "synthetic",
            "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": f"{n}^3 interior cells, 2 ghost layers (periodic x,y), the reference driver's "
                                   f"STZ parameters and quasi-static step dt = {dt}, velocities N(0,1e-3), stress "
                                   "magnitudes sbar ~ U(0.5, 1.15) sy (seed 0); inputs (2.6 GB) larger than L2",
                       "plastic_fraction": plastic, "yielded": yielded},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "bytes_per_cell": ADV_BYTES_PER_CELL, "peak_kind": kind},
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 8 * npts * len(ins),
                    "d2h_bytes_per_step": 8 * npts * len(advect.OUTPUTS)},
            "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": 1, "kind": "port",
                             "sample": f"C restatement of the step on {m}^3 cells of the same kind, scaled by cell count"},
            "gpu_launches": 3 * args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, choices=[2, 3, 5, 6, 7], default=2,
                    help="2: the 256x256x257 headline solve (default); 3: 512x512x257 variable mu, mixed vs FP64; "
                         "5: 50-solve sequence with checkpointed backward; 6: per-step coefficient change; "
                         "7: the quasi-static advection step on 256^3 cells")
    ap.add_argument("--cells", type=int, default=256, help="cells per dimension of the advection workload (--config 7)")
    ap.add_argument("--v-down", type=int, default=V_DOWN, help="sweeps before the coarse-grid correction")
    ap.add_argument("--v-up", type=int, default=V_UP, help="sweeps after it")
    ap.add_argument("--sweep-growth", type=int, choices=[0, 1], default=0,
                    help="1: v_down + i / v_up + i - 1 sweeps on level i, as the reference")
    ap.add_argument("--max-coarse", type=int, default=1024,
                    help="hierarchy stop rule of the headline solve (reference: 1024 nodes)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.config == 3 and args.impl == "ours":
        run_config3(args, local)
    elif args.config == 5 and args.impl == "ours":
        run_config5(args, local)
    elif args.config == 6 and args.impl == "ours":
        run_coeff_change(args, local)
    elif args.config == 7 and args.impl == "ours":
        run_advection(args, local, n=args.cells)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
