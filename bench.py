#!/usr/bin/env python
"""Benchmark: time to 1e-8 relative residual on the 256^3 periodic 12th-order
Poisson problem with AAR (omega = beta = 0.6, m = 7, p = 6), mixed precision
(FP32 inner AAR inside FP64 residual refinement) against plain FP64, on one
GB300, plus the achieved HBM bandwidth of the dominant kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl lsg|reference]

A step is one complete solve from x0 = 0.  Inputs live in HBM before the
timed region; every solve streams ~17 vectors of 67-134 MB, far more than the
129 MB L2, so no flush is needed between steps.  For N > 1 (torchrun) each
rank solves its own copy of the problem (replicas; the path has no data
exchange on one GPU per rank), and the time is the max over ranks.

--impl reference times the CPU implementation of the same path on the host
cores: the C restatement of the reference solver (oracle/), run with every
host thread on a bounded sample of iterations of the same problem and
extrapolated to the iteration count the full solve needs.  --cpu-full runs
one complete CPU solve instead (about 2.5 minutes on 16 cores) to check that
extrapolation.

Every solution on the line carries its error against the FFT diagonal solve
of the periodic operator (an exact FP64 solve, mean removed), computed here
with torch's FFT from the operator's coefficients.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "linear-solver_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_GRID = 256
SEED = 1
SOLVER_KW = dict(omega=0.6, beta=0.6, m=7, p=6, tol=1e-8)
METRIC = "time to 1e-8 rel. residual, 256^3 Poisson AAR: mixed vs FP64 on GB300; HBM GB/s"
WORKLOAD = ("256^3 periodic 12th-order FD Poisson (a = -1/(4 pi), FDn = 6, Jacobi), AAR m=7 p=6 "
            "omega=beta=0.6, tol 1e-8, b ~ U[-0.5,0.5] seed 1 mean-free, x0 = 0")
# Iterations the FP64 AAR needs on this workload (the reference's algorithm;
# the CPU oracle and the GPU FP64 solver agree).  Used to extrapolate the
# bounded CPU sample.
LARGE_GOLDEN = os.path.join(ROOT, "tests", "golden", "large_256.json")
CPU_SAMPLE_ITERS = 24
# DRAM bytes (read + write) of one launch of the dominant kernel at this
# workload, from an ncu capture of that kernel on this workload (a constant:
# the timed run is not captured); keyed by "residual ring in use".
RICH32_TRAFFIC_BYTES = {False: 224.2e6, True: 101.0e6}


def solve_roofline(n, inner_iters, outer_iters, seconds, fp64_iters, fp64_seconds, peak):
    """Algorithmic bytes of a whole AAR solve (11 vectors per iteration at
    m = 7, p = 6: (p - 1) 7-vector Richardson steps and one (3m + 10)-vector
    extrapolation per cycle; 5 FP64 vectors per mixed outer step) over its
    wall time, for the mixed and the FP64 solve."""
    per_it = ((SOLVER_KW["p"] - 1) * 7 + 3 * SOLVER_KW["m"] + 10) / SOLVER_KW["p"]
    mixed_b = per_it * n * 4 * inner_iters + 5 * 8 * n * outer_iters
    fp64_b = per_it * n * 8 * fp64_iters
    return {"vectors_per_iteration": per_it, "unit": "GB/s", "peak": peak,
            "mixed": {"bytes": mixed_b, "achieved": mixed_b / seconds / 1e9, "frac": mixed_b / seconds / 1e9 / peak},
            "fp64": {"bytes": fp64_b, "achieved": fp64_b / fp64_seconds / 1e9,
                     "frac": fp64_b / fp64_seconds / 1e9 / peak},
            "note": "the reference algorithm's data movement; the residual ring moves ~34 vectors per "
                    "6-iteration cycle instead of 66, so the mixed figure can exceed the copy peak"}


def aar_form_in_use(lsg):
    """The FP32 AAR form the library will run (0 ring, 1 lean, 2 x-carrying)."""
    f = lsg.set_aar_form(0)
    lsg.set_aar_form(f)
    return f
FP64_SOLVERS = ("aar", "pgr", "pl2r", "cg")


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(v: float, ws: int) -> float:
    """The slowest rank's time (every rank gets it)."""
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _large_iters(solver: str = "aar"):
    try:
        with open(LARGE_GOLDEN) as f:
            return int(json.load(f)[solver]["iters"])
    except Exception:
        return None


def cpu_sample(iters_full: int, threads: int | None = None, solver: str = "aar", full: bool = False):
    """Times CPU_SAMPLE_ITERS iterations (or, full=True, the whole solve) of
    the oracle solver on the full workload with every host thread; returns
    (seconds to solution, seconds/iter, threads, iterations timed).  The
    oracle's work arrays are first-touched before its timer starts, so the
    sample measures the steady state."""
    import workloads
    from oracle import oracle as O

    O.build(with_ref=False)
    threads = threads or O.lib().lsgo_max_threads()
    b = workloads.uniform_rhs(N_GRID, SEED)
    kw = dict(SOLVER_KW)
    if solver != "aar":
        kw.pop("beta")
    _, r = O.solve(solver, b, None, max_iter=100000 if full else CPU_SAMPLE_ITERS, threads=threads, **kw)
    timed = r["iters"] if full else CPU_SAMPLE_ITERS
    per_iter = r["seconds"] / max(timed, 1)
    return (r["seconds"] if full else per_iter * iters_full), per_iter, threads, timed


def fft_reference(b, op):
    """The exact FP64 solution of the periodic operator (its DFT symbol is
    a (3 c_0 + sum_p 2 c_p (cos 2 pi p kx/nx + cos .. ky + cos .. kz)) + sigma),
    mean-free for the singular Poisson case; torch FFT on the device."""
    import math

    import torch
    nz, ny, nx = b.shape
    c = op.coeff

    def axis(n):
        k = torch.arange(n, dtype=torch.float64, device=b.device)
        s = torch.zeros(n, dtype=torch.float64, device=b.device)
        for p in range(1, op.radius + 1):
            s += 2.0 * c[p] * torch.cos(2.0 * math.pi * p * k / n)
        return s

    lam = op.a * (3.0 * c[0] + axis(nz)[:, None, None] + axis(ny)[None, :, None] + axis(nx)[None, None, :])
    lam = lam + op.sigma
    bh = torch.fft.fftn(b)
    singular = op.sigma == 0  # the constant mode (its symbol is zero up to rounding)
    if singular:
        lam[0, 0, 0] = 1.0
    xh = bh / lam
    if singular:
        xh[0, 0, 0] = 0.0
    x = torch.fft.ifftn(xh)
    return x.real if not torch.is_complex(b) else x


def err_vs_fft(x, xf, mean_free=True):
    """Relative 2-norm error of x against the FFT solution (means removed for
    the singular Poisson operator)."""
    if mean_free:
        x = x - x.mean()
    return ((x - xf).norm() / xf.norm()).item()


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    iters = _large_iters()
    if iters is None:
        print(json.dumps({"impl": "reference", "unavailable": "iteration count of the 256^3 "
                          "workload not pinned (tests/golden/large_256.json missing)"}))
        return 0
    samples = []
    threads = None
    for i in range(args.warmup + args.steps):
        tts, per_iter, threads, _ = cpu_sample(iters)
        if i >= args.warmup:
            samples.append(tts)
    value = statistics.mean(samples)
    sample = (f"{CPU_SAMPLE_ITERS} of {iters} AAR iterations at 256^3 per step (work arrays "
              f"first-touched before the timer), extrapolated by the iteration count; {threads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "n": N_GRID, "solver": "AAR FP64",
                                         "implementation": "C restatement of MPI_REAL AAR (oracle/), OpenMP"},
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port", "sample": sample,
                         "extrapolated_from": f"{CPU_SAMPLE_ITERS} iterations x {iters} / {CPU_SAMPLE_ITERS}"},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_lsg(args):
    import numpy as np
    import torch

    import lsg
    import workloads

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = N_GRID
    op = lsg.Operator(n)
    bh = workloads.uniform_rhs(n, SEED)
    b = torch.from_numpy(bh).to(dev)
    N = n ** 3
    stream = torch.cuda.current_stream()

    def solve_mixed():
        return lsg.aar_mixed(op, b, **SOLVER_KW)

    def solve_fp64():
        return lsg.aar(op, b, **SOLVER_KW)

    # ---- launch-shape autotuning (Richardson pass of both precisions), then
    # warm-up (also builds the work arrays); both outside the timed region
    tuned = {"f32": lsg.autotune(op, torch.float32), "f64": lsg.autotune(op, torch.float64)}
    for _ in range(args.warmup):
        x, info = solve_mixed()
    torch.cuda.synchronize()

    # ---- timed region: K mixed solves (no per-launch profiling events inside)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    infos = []
    with ClockSampler(local) as clk:
        _barrier(ws)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            x, info = solve_mixed()
            infos.append(info)
        e1.record(stream)
        torch.cuda.synchronize()
        _barrier(ws)
    # ---- one more solve with CUDA events around every launch (per-kernel
    # device times for the roofline), outside the timed region
    lsg.profile(True)
    solve_mixed()
    torch.cuda.synchronize()
    lsg.profile(False)
    prof = lsg.profile_read()
    ms = e0.elapsed_time(e1) / args.steps
    ms = _max_over_ranks(ms, ws)
    value = ms / 1e3
    true_res = ((b - lsg.apply(op, x)).norm() / b.norm()).item()
    xf = fft_reference(b, op)
    err_mixed = err_vs_fft(x, xf)

    # ---- the four FP64 solvers (the drop-in's arithmetic: double-float
    # stencil sums at this tolerance) and the FP64 AAR in FP64 arithmetic
    def timed_solve(fn):
        fn()
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        xs, inf = fn()
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / 1e3, xs, inf

    fp64 = {}
    for s in FP64_SOLVERS:
        kw = dict(SOLVER_KW)
        if s != "aar":
            kw.pop("beta")
        secs, xs, inf = timed_solve(lambda: lsg.SOLVERS[s](op, b, **kw))
        fp64[s] = {"seconds": secs, "iters": inf["iters"], "relres": inf["relres"],
                   "true_relres": ((b - lsg.apply(op, xs)).norm() / b.norm()).item(),
                   "err_vs_fft": err_vs_fft(xs, xf), "status": inf["status_name"],
                   "updates_per_s": N * inf["iters"] / secs}
        if s == "aar":
            x64 = xs
    fp64_s = fp64["aar"]["seconds"]
    prev = lsg.set_fp64_arith(1)
    secs, xs, inf = timed_solve(solve_fp64)
    lsg.profile(True)
    lsg.aar(op, b, max_iter=60, **SOLVER_KW)
    torch.cuda.synchronize()
    lsg.profile(False)
    prof64x = lsg.profile_read()
    lsg.set_fp64_arith(prev)
    fp64_exact = {"seconds": secs, "iters": inf["iters"], "relres": inf["relres"],
                  "err_vs_fft": err_vs_fft(xs, xf)}
    del xs
    # per-kernel times of the FP64 iteration: 60 profiled iterations
    lsg.profile(True)
    lsg.aar(op, b, max_iter=60, **{k: v for k, v in SOLVER_KW.items()})
    torch.cuda.synchronize()
    lsg.profile(False)
    prof64 = lsg.profile_read()

    # ---- end to end: the reference-prototype AAR(POISSON*, ...) on pinned host
    # buffers (H2D of x0 and rhs, D2H of x inside the timed region), mixed mode
    xh = torch.zeros((n, n, n), dtype=torch.float64).pin_memory()
    rh = torch.from_numpy(bh).pin_memory()
    lsg.set_compat_mode(True)
    xh.zero_()
    lsg.compat_solve("aar", xh.numpy(), rh.numpy(), **SOLVER_KW)  # warm the staging buffers
    e2e = []
    for _ in range(args.steps):
        xh.zero_()
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        ri = lsg.compat_solve("aar", xh.numpy(), rh.numpy(), **SOLVER_KW)
        c1.record(stream)
        torch.cuda.synchronize()
        e2e.append(c0.elapsed_time(c1) / 1e3)
    lsg.set_compat_mode(False)
    e2e_s = _max_over_ranks(statistics.mean(e2e), ws)
    e2e_ok = ri["status"] == 0

    # ---- roofline of the dominant kernel (FP32 fused Richardson step)
    peak, peak_kind = _peaks()
    rl, rms = prof["richardson"]
    rich_ms = rms / max(rl, 1)
    # the FP32 inner solver's Richardson pass: in the residual-ring form it
    # reads r_{k-1} (stencil) and writes r_k; the lean form also writes the H
    # and DF columns
    ring = aar_form_in_use(lsg) == 0
    rich_bytes = (2 if ring else 4) * N * 4
    achieved = rich_bytes / (rich_ms * 1e-3) / 1e9
    total_ms = sum(v[1] for v in prof.values())
    r64l, r64ms = prof64["richardson"]
    rich64_ms = r64ms / max(r64l, 1)
    r64xl, r64xms = prof64x["richardson"]
    rich64x_ms = r64xms / max(r64xl, 1)
    rich64_bytes = 7 * N * 8  # reads x, r, b; writes x', r', H, DF

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        iters_full = fp64["aar"]["iters"]
        tts, per_iter, threads, timed = cpu_sample(iters_full, full=args.cpu_full)
        cpu = {"value": tts, "unit": "s", "cores": threads, "kind": "port",
               "sample": (f"one full {timed}-iteration AAR solve of the same 256^3 workload on {threads} threads"
                          if args.cpu_full else
                          f"{CPU_SAMPLE_ITERS} of {iters_full} AAR iterations of the same 256^3 workload on "
                          f"{threads} threads (work arrays first-touched before the timer), extrapolated by the "
                          f"iteration count"),
               "measured": bool(args.cpu_full), "seconds_per_iter": per_iter}
        # the other FP64 solvers: seconds per iteration on the same cores (bounded samples)
        per = {}
        for s in FP64_SOLVERS:
            if s == "aar":
                per[s] = per_iter
                continue
            _, pi, _, _ = cpu_sample(fp64[s]["iters"], threads=threads, solver=s)
            per[s] = pi
        for s in FP64_SOLVERS:
            fp64[s]["cpu_seconds_per_iter"] = per[s]
            fp64[s]["cpu_seconds_extrapolated"] = per[s] * fp64[s]["iters"]

    extra = other_workloads(dev) if (rank == 0 and not args.no_extra) else None

    launches = sum(i["launches"] for i in infos)
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 inner / f64 refinement", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "solver": "AAR mixed (lsg_aar_mixed)",
                   "l2": "no flush: each solve streams ~17 vectors of 67-134 MB (> 129 MB L2)",
                   "parallelism": f"replicas x{ws}",
                   "autotuned_richardson": {k: {kk: v[kk] for kk in ("threads_y", "rows_per_thread", "lz",
                                                                       "us_best", "us_default")}
                                            for k, v in tuned.items()}},
        "mixed": {"inner_iters": infos[-1]["inner_iters"], "outer_iters": infos[-1]["outer_iters"],
                  "relres": infos[-1]["relres"], "true_relres_fp64": true_res, "err_vs_fft": err_mixed},
        "fp64": {"seconds": fp64_s, "iters": fp64["aar"]["iters"], "relres": fp64["aar"]["relres"],
                 "true_relres": fp64["aar"]["true_relres"], "err_vs_fft": fp64["aar"]["err_vs_fft"],
                 "speedup_mixed_vs_fp64": fp64_s / value,
                 "stencil_arith": "double-float sums on the FP32 pipe (FP64 storage and epilogue)",
                 "richardson_ms": rich64_ms,
                 "richardson_gpts": N / (rich64_ms * 1e-3) / 1e9,
                 "fp64_arith": dict(fp64_exact, richardson_ms=rich64x_ms)},
        "fp64_solvers": fp64,
        "roofline_fp64": {"kernel": "stencil_kernel<double, RichOp, double-float> (fused FP64 Richardson step)",
                          "bytes_per_launch": rich64_bytes, "avg_launch_ms": rich64_ms,
                          "achieved": rich64_bytes / (rich64_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                          "frac": rich64_bytes / (rich64_ms * 1e-3) / 1e9 / peak,
                          "frac_fp64_arith": rich64_bytes / (rich64x_ms * 1e-3) / 1e9 / peak,
                          "bound": "issue (double-float arithmetic, ~950 instructions per point)"},
        "roofline": {"bound": "hbm",
                     "kernel": ("stencil_x2_kernel<float, RichRingOp> in the tuned paired shape (Richardson step of "
                                "the residual ring: r_k only)" if ring else
                                "stencil_x2_kernel<float, RichLeanOp> in the tuned paired shape (fused Richardson "
                                "step, x left out)"),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
                     "traffic": RICH32_TRAFFIC_BYTES[ring], "traffic_unit": "bytes per launch (ncu)",
                     "traffic_source": "constant from an ncu capture of this kernel on this workload, not of this run",
                     "bytes_per_launch": rich_bytes, "avg_launch_ms": rich_ms,
                     "note": ("residual ring: 2 vectors per launch (the H and DF columns are rebuilt from "
                              "consecutive residuals by the Gram and update kernels; the lean form moved 4, the "
                              "x-carrying form 6)" if ring else
                              "lean form: 4 vectors per launch (x left out; the x-carrying form moved 6)"),
                     "share_of_kernel_time": rms / total_ms if total_ms else None},
        "kernel_profile_ms": {k: round(v[1], 4) for k, v in prof.items() if v[0]},
        "updates_per_s": {"mixed": N * infos[-1]["inner_iters"] / value, "fp64": N * fp64["aar"]["iters"] / fp64_s},
        # whole-solve figure: the reference algorithm's data movement (AAR average
        # 11 N s per iteration at m = 7, p = 6; a mixed solve's outer step adds
        # 5 N 8 bytes) over the measured solve time
        "roofline_solve": solve_roofline(N, infos[-1]["inner_iters"], infos[-1]["outer_iters"], value,
                                         fp64["aar"]["iters"], fp64_s, peak),
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": 2 * N * 8,
                "d2h_bytes_per_step": N * 8, "path": "AAR(POISSON*, ...) drop-in, mixed mode, pinned host buffers",
                "converged": e2e_ok},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "other_workloads": extra,
    }
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def other_workloads(dev):
    """One timed run each of the other measured workloads (inputs resident,
    one warm-up run first): 384^3 mixed AAR to 1e-10 on the 64-blob rhs; 48
    batched complex shifted-Helmholtz solves (sides 32..160, complex64 inner
    / complex128 refinement, tol 1e-8); the differentiable batch of 16 real
    128^3 solves (mixed forward to 1e-9 + adjoint backward); GMRES(30), CG
    and AAR on the 256^3 workload at 1e-6."""
    import numpy as np
    import torch

    import lsg
    import workloads

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, out

    res = {}
    n = 384
    op = lsg.Operator(n)
    b = torch.from_numpy(workloads.blob_rhs(n, 3)).to(dev)
    secs, (x, r) = timed(lambda: lsg.aar_mixed(op, b, tol=1e-10))
    res["blobs_384_mixed_1e-10"] = {"seconds": secs, "inner_iters": r["inner_iters"],
                                    "outer_iters": r["outer_iters"], "relres": r["relres"],
                                    "true_relres_fp64": ((b - lsg.apply(op, x)).norm() / b.norm()).item(),
                                    "err_vs_fft": err_vs_fft(x, fft_reference(b, op)),
                                    "updates_per_s": n ** 3 * r["inner_iters"] / secs}
    del b, x
    batch = workloads.helmholtz_batch(2024)
    ops = [lsg.Operator(m, a=-float(m * m), sigma=s) for m, s, _ in batch]
    bs = [torch.from_numpy(v).to(dev) for _, _, v in batch]
    secs, (xs, rs) = timed(lambda: lsg.aar_batched(ops, bs, mixed=True, tol=1e-8))
    pts = sum(m ** 3 * r["iters"] for (m, _, _), r in zip(batch, rs))
    errs = [err_vs_fft(xi, fft_reference(bi, oi), mean_free=False) for xi, bi, oi in zip(xs, bs, ops)]
    res["helmholtz_48_batched"] = {"seconds": secs, "instances": len(batch), "err_vs_fft_max": max(errs),
                                   "converged": sum(r["status"] == 0 for r in rs),
                                   "iters_min": min(r["iters"] for r in rs),
                                   "iters_max": max(r["iters"] for r in rs),
                                   "updates_per_s": pts / secs, "launches": rs[0]["launches"]}
    del bs, xs
    probs = workloads.differentiable_batch(5)
    bb = torch.stack([torch.from_numpy(v[1]) for v in probs]).to(dev)
    xstar = torch.stack([torch.from_numpy(v[2]) for v in probs]).to(dev)
    sig = torch.tensor([v[0] for v in probs], dtype=torch.float64, device=dev)

    def fwd_bwd():
        bq = bb.clone().requires_grad_(True)
        sq = sig.clone().requires_grad_(True)
        x = lsg.solve_shifted(bq, sq, a=-128.0 * 128.0, precision="mixed", tol=1e-9)
        (0.5 * ((x - xstar) ** 2).sum()).backward()
        return sq.grad

    secs, _ = timed(fwd_bwd)
    res["differentiable_16x128_fwd_bwd"] = {"seconds": secs}
    del bb, xstar
    # the reference's KSP comparison (PETSC_REAL/main.c:84-184): GMRES(30) and CG
    # against AAR at PETSc's tolerance 1e-6, FP64, the 256^3 workload
    op = lsg.Operator(N_GRID)
    b = torch.from_numpy(workloads.uniform_rhs(N_GRID, SEED)).to(dev)
    cmp = {}
    for name, fn in (("gmres30", lambda: lsg.gmres(op, b, restart=30, tol=1e-6, max_iter=20000)),
                     ("cg", lambda: lsg.cg(op, b, tol=1e-6)),
                     ("aar_fp64", lambda: lsg.aar(op, b, tol=1e-6)),
                     ("aar_mixed", lambda: lsg.aar_mixed(op, b, tol=1e-6))):
        secs, (x, r) = timed(fn)
        cmp[name] = {"seconds": secs, "iters": r["iters"], "relres": r["relres"], "status": r["status_name"]}
    res["krylov_comparison_256_1e-6"] = cmp
    # the complex comparison (PETSC_COMPLEX/main.c:47-175: AAR against GMRES,
    # LGMRES and BiCG): one 96^3 shifted Helmholtz instance, sigma = 20 + 10i,
    # complex128, 1e-6
    n = 96
    rng = np.random.default_rng(96)
    bc = torch.from_numpy(rng.uniform(-0.5, 0.5, (n, n, n)) + 1j * rng.uniform(-0.5, 0.5, (n, n, n))).to(dev)
    opc = lsg.Operator(n, a=-float(n * n), sigma=20 + 10j)
    xfc = fft_reference(bc, opc)
    ccmp = {}
    for name, fn in (("aar", lambda: lsg.aar(opc, bc, tol=1e-6)),
                     ("aar_mixed", lambda: lsg.aar_mixed(opc, bc, tol=1e-6)),
                     ("gmres30", lambda: lsg.gmres(opc, bc, restart=30, tol=1e-6, max_iter=20000)),
                     ("lgmres30_2", lambda: lsg.lgmres(opc, bc, restart=30, aug=2, tol=1e-6, max_iter=20000)),
                     ("cocg", lambda: lsg.cocg(opc, bc, tol=1e-6))):
        secs, (x, r) = timed(fn)
        ccmp[name] = {"seconds": secs, "iters": r["iters"], "relres": r["relres"], "status": r["status_name"],
                      "err_vs_fft": err_vs_fft(x, xfc, mean_free=False)}
    res["helmholtz_krylov_comparison_96_1e-6"] = ccmp
    # block-Jacobi ICC(0) AAR (the reference's pc = 1) against Jacobi on the 256^3 workload
    op = lsg.Operator(N_GRID)
    b = torch.from_numpy(workloads.uniform_rhs(N_GRID, SEED)).to(dev)
    icc = {}
    for name, fn in (("jacobi", lambda: lsg.aar(op, b, **SOLVER_KW)),
                     ("icc0_8x8x8", lambda: lsg.aar_icc(op, b, block=(8, 8, 8), **SOLVER_KW))):
        secs, (x, r) = timed(fn)
        icc[name] = {"seconds": secs, "iters": r["iters"], "relres": r["relres"], "status": r["status_name"]}
    res["aar_fp64_icc0_vs_jacobi_256"] = icc
    return res


def run_case(case: str, tune_file=None):
    """Short fixed invocations for profilers (ncu): one launch pattern each.

    rich32 / rich64: 6 AAR iterations (FP32 / FP64 vectors) of the 256^3
    workload -- the initial residual, five fused Richardson steps and one
    Anderson step (Gram, m x m solve, update, residual).
    mixed / fp64: one complete solve of the benchmark workload.
    helmholtz: the 48-instance complex shifted-Helmholtz batch (mixed, tol
    1e-8) twice, a warm-up and the one in the "solve" range.
    icc: the first three iterations of the block-Jacobi ICC(0) AAR (8^3
    boxes) at 128^3 (FP64, default launch shapes).
    Launch shapes are autotuned first, as in the benchmark run.  tune_file:
    when it exists, the shapes are read from it instead (a profiler slows
    every launch, the tuner's timings too); otherwise they are tuned and
    saved there, so a plain run followed by the profiled run of the same
    command profiles the plain run's shapes.
    """
    import torch

    import lsg
    import workloads

    torch.cuda.set_device(0)
    if case == "helmholtz":
        batch = workloads.helmholtz_batch(2024)
        ops = [lsg.Operator(m, a=-float(m * m), sigma=s) for m, s, _ in batch]
        bs = [torch.from_numpy(v).cuda() for _, _, v in batch]
        lsg.aar_batched(ops, bs, mixed=True, tol=1e-8)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("solve")
        xs, rs = lsg.aar_batched(ops, bs, mixed=True, tol=1e-8)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"case": case, "instances": len(rs), "iters_max": max(r["iters"] for r in rs),
                          "seconds": rs[0]["seconds"], "launches": rs[0]["launches"],
                          "converged": sum(r["status"] == 0 for r in rs)}))
        return 0
    if case == "icc":
        op = lsg.Operator(128)
        b = torch.from_numpy(workloads.uniform_rhs(128, 1)).cuda()
        x, info = lsg.aar_icc(op, b, block=(8, 8, 8), max_iter=3, tol=1e-8)
        torch.cuda.synchronize()
        print(json.dumps({"case": case, "iters": info["iters"], "status": info["status_name"]}))
        return 0
    op = lsg.Operator(N_GRID)
    b = torch.from_numpy(workloads.uniform_rhs(N_GRID, SEED)).cuda()
    if tune_file and os.path.exists(tune_file):
        lsg.autotune_load(tune_file)
    else:
        lsg.autotune(op, torch.float32 if case in ("rich32", "mixed") else torch.float64)
        if tune_file:
            lsg.autotune_save(tune_file)
    torch.cuda.synchronize()
    # the solve's launches sit in an NVTX range "solve" (ncu --nvtx
    # --nvtx-include "solve/" leaves out the tuner's launches)
    torch.cuda.nvtx.range_push("solve")
    if case == "rich32":
        x, info = lsg.aar(op, b.float(), max_iter=6, **SOLVER_KW)
    elif case == "rich64":
        x, info = lsg.aar(op, b, max_iter=6, **SOLVER_KW)
    elif case == "mixed":
        x, info = lsg.aar_mixed(op, b, **SOLVER_KW)
    else:
        x, info = lsg.aar(op, b, **SOLVER_KW)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"case": case, "iters": info["iters"], "relres": info["relres"],
                      "launches": info["launches"], "status": info["status_name"]}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lsg", choices=["lsg", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extra", action="store_true", help="skip the other measured workloads")
    ap.add_argument("--cpu-full", action="store_true",
                    help="time one complete CPU solve for the baseline instead of a bounded sample")
    ap.add_argument("--case", choices=["rich32", "rich64", "mixed", "fp64", "helmholtz", "icc"],
                    help="run one short fixed invocation for a profiler and exit")
    ap.add_argument("--tune-file", help="--case: launch shapes read from this file if it exists, else saved there")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case, args.tune_file)
    if args.impl == "reference":
        return run_reference(args)
    return run_lsg(args)


if __name__ == "__main__":
    sys.exit(main())
