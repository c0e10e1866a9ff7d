"""Benchmark: time to a 1e-10 relative residual on one GB300.

Workload (one "step" = one complete preconditioned solve of one system):
  3D 7-point first-order upwind convection-diffusion, 128^3 grid
  (n = 2,097,152, nnz = 14,581,760), cell Peclet 10, velocity (1, .5, .25);
  b ~ N(0,1) seed 0, x0 = 0; ParILU(0) with 3 synchronous sweeps from the
  A-initial guess; FGMRES-Householder(50) restarted, right-preconditioned by
  exact (sync-free) triangular solves; stop at ||r|| <= 1e-10 ||r0||.
Headline arm: FP32 factors and solves inside the FP64 FGMRES ("mixed");
the all-FP64 GPU path is timed beside it.

`value` is device time per solve with A resident in HBM (CUDA events on the
solver stream).  `e2e` is the same solve through the LACE-named C ABI
(data_PariLU_v0_3_prescribedSweeps + data_fgmres_householder_restart) from
host buffers, copies included.  `--impl reference` times the CPU
restatement of LACE's path (the oracle port; LACE's own build needs MKL
and the LACE tree, neither of which exists on the GPU host) on all host
cores.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = 128
SWEEPS = 3
M = 50
RTOL = 1e-10
RESTART_MAX = 20
METRIC = "solve s to 1e-10 resid, mixed-prec vs FP64 on 1 GB300; SpMV/SpTRSV HBM GB/s"
WORKLOAD = (f"convdiff3d {GRID}^3 7-pt upwind Pe10 (n={GRID**3}, nnz=14581760), ParILU(0) {SWEEPS} sync sweeps, "
            f"FGMRES-Householder({M}) to 1e-10 rel, b~N(0,1) seed 0, x0=0")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float) -> float:
    """The slowest rank's value (each rank times its own replica); the
    reduction tensor lives where the process group's backend works (the GPU
    for NCCL, the host for gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def build_problem(grid: int = GRID):
    from lace_gb300 import problems as P
    A = P.convdiff3d(grid)
    b = P.rhs_normal(A.n, 0)
    return A, b


def algorithmic_bytes(A, nnzL, nnzU, prec: str):
    """Compulsory bytes: each CSR array of the triangle or operator read once
    (int32 indices), each vector read or written once.  Per unit (one row):
    L: (nnzL/n - 1) off-diagonal values + columns, a row pointer, q and t;
    U: the same plus the diagonal value, t and z."""
    n = A.n
    sv = 4 if prec != "fp64" else 8   # factor value and solve-vector bytes
    sx = sv
    bl = (nnzL - n) * (sv + 4) + n * 4 + n * sx + n * sx
    bu = (nnzU - n) * (sv + 4) + n * (4 + sv) + n * sx + n * sx
    spmv = A.nnz * (8 + 4) + n * (4 + 8 + 8)
    return {"sptrsv_L": bl, "sptrsv_U": bu, "sptrsv_pair": bl + bu, "spmv": spmv}


STEP_J = 15  # the Arnoldi step the roofline is quoted on (16 basis columns)


def step_bytes(A, j: int) -> int:
    """Compulsory bytes of one one-kernel Householder step j in mixed
    precision (w stays in shared memory): the operator's CSR arrays and z
    (FP32) once, the j+1 basis columns once in FP64 (V^T w and w -= V y) and
    once in FP32 (q = e - V c), and the writes: the new column in FP64 and
    FP32, q, and the two solve outputs marked unsolved (FP32)."""
    n = A.n
    return (A.nnz * (8 + 4) + (n + 1) * 4 + n * 4 + (j + 1) * n * (8 + 4) + n * (8 + 4 + 4 + 4 + 4))


def profiled_traffic(path: str, key: str):
    """DRAM bytes (read + write) per launch from a committed ncu summary, or None."""
    try:
        for line in open(os.path.join(ROOT, "profiles", path)):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def run_ours(args):
    import torch

    import lace_gb300 as lg
    from lace_gb300 import dropin

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    A, b = build_problem(args.grid if (args.only_mgs or args.only_householder) else GRID)
    stream = torch.cuda.Stream()
    ctx = lg.Context(local, stream=stream)
    ctx.upload(A)
    bd = torch.tensor(b, dtype=torch.float64, device="cuda")
    xd = torch.zeros(A.n, dtype=torch.float64, device="cuda")

    pin = {}
    if args.trsv_schedule:
        R, cpb, w, cl = (int(v) for v in args.trsv_schedule.split(","))
        pin = {"rows_per_lane": R, "schedule": (cpb, w, cl)}

    def solve(prec, orth="householder"):
        ctx.set_options(precision=prec, **pin)
        with torch.cuda.stream(stream):
            xd.zero_()
        ctx.parilu0(SWEEPS)
        return ctx.fgmres(bd, xd, search_max=M, restart_max=RESTART_MAX, rtol=RTOL, orthogonalization=orth)

    def timed(prec, k, w, orth="householder"):
        for _ in range(w):
            solve(prec, orth)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        times = []
        res = None
        t0 = time.perf_counter()
        for _ in range(k):
            ev0.record(stream)
            res = solve(prec, orth)
            ev1.record(stream)
            ev1.synchronize()
            times.append(ev0.elapsed_time(ev1) / 1e3)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if world > 1:
            torch.distributed.barrier()
        return times, wall, res

    if args.only_mgs or args.only_householder:
        # profiling aid: one solve kind alone (no contract line)
        orth = "mgs" if args.only_mgs else "householder"
        t_one, _, r_one = timed("fp32", args.steps, args.warmup, orth)
        if rank == 0:
            print(json.dumps({orth: {"value": statistics.median(t_one), "unit": "s",
                                     "iterations": r_one.total_iterations}}))
        ctx.close()
        return

    with ClockSampler(local) as clk:
        t_mixed, wall_mixed, r_mixed = timed("fp32", args.steps, args.warmup)
    clocks = clk.summary()
    x_mixed = xd.cpu().numpy()
    t_fp64, wall_fp64, r_fp64 = timed("fp64", max(2, args.steps // 2), 1)
    x_fp64 = xd.cpu().numpy()
    # the same solve with LACE's other Krylov solver, FGMRES with modified
    # Gram-Schmidt (data_fgmres_restart), mixed precision
    t_mgs, wall_mgs, r_mgs = timed("fp32", max(2, args.steps // 2), 1, "mgs")
    x_mgs = xd.cpu().numpy()

    def true_rel(x):
        return float(np.linalg.norm(b - A.matvec(x)) / np.linalg.norm(b))

    # ---- dominant kernel: the preconditioner pair of one FGMRES step (fill +
    # L solve + fill + U solve, FP32 vectors), enqueued back to back on the
    # solver stream and timed there with CUDA events
    ctx.set_options(precision="fp32", **pin)
    ctx.parilu0(SWEEPS)
    q = torch.randn(A.n, dtype=torch.float64, device="cuda")
    z = torch.empty_like(q)
    ctx.apply_precond(q, z)  # plans, schedule and values in place
    q32 = q.float()
    z32 = torch.empty_like(q32)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("sptrsv_pair")  # ncu --nvtx-include "sptrsv_pair/" selects these launches
    for _ in range(3):
        ctx.precond_enqueue(q32, z32)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    reps = 20
    ev0.record(stream)
    for _ in range(reps):
        ctx.precond_enqueue(q32, z32)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.nvtx.range_pop()
    trsv_s = ev0.elapsed_time(ev1) / 1e3 / reps
    ctx.apply_precond(q, z)  # surfaces a spin-wait timeout of the timed pairs, if any
    sched = dict(zip(("rows_per_lane", "chunks_per_block", "warps", "cluster"), ctx.trsv_schedule()))
    # SpMV (FP64 operator) alone
    y = torch.empty_like(q)
    for _ in range(3):
        ctx.spmv(q, y)
    ev0.record(stream)
    for _ in range(reps):
        ctx.spmv(q, y)
    ev1.record(stream)
    ev1.synchronize()
    spmv_s = ev0.elapsed_time(ev1) / 1e3 / reps
    Lp = np.diff(A.row)
    nnzL = int(np.sum(A.col <= np.repeat(np.arange(A.n), Lp)))
    nnzU = int(np.sum(A.col >= np.repeat(np.arange(A.n), Lp)))
    ab = algorithmic_bytes(A, nnzL, nnzU, "fp32")
    traffic_pair = profiled_traffic("sptrsv_pair_convdiff128.txt", "dram_bytes_per_pair")
    # ---- the dominant kernel: the one-kernel Arnoldi step (Householder),
    # replayed at step STEP_J on the basis of the last mixed-precision solve
    ctx.set_options(precision="fp32", **pin)
    ctx.parilu0(SWEEPS)
    with torch.cuda.stream(stream):
        xd.zero_()
    ctx.fgmres(bd, xd, search_max=M, restart_max=RESTART_MAX, rtol=RTOL)
    step_s = ctx.time_arnoldi_step("householder", j=STEP_J, reps=20)
    sb = step_bytes(A, STEP_J)
    step_gbs = sb / step_s / 1e9
    traffic = args.traffic if args.traffic is not None else profiled_traffic(
        "arnoldi_step_convdiff128.txt", "dram_bytes_per_launch")
    trsv_gbs = ab["sptrsv_pair"] / trsv_s / 1e9
    spmv_gbs = ab["spmv"] / spmv_s / 1e9

    # ---- e2e: the LACE-named C ABI from host buffers (copies inside)
    e2e = None
    if not args.skip_e2e:
        dropin.set_options(precision="fp32")
        Am = dropin.csr(A.row, A.col, A.val, A.n)
        e2e_times = []
        for it in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            L, U, info = dropin.parilu_mats(Am, max_sweeps=SWEEPS)
            x, rc, glog = dropin.fgmres_householder_restart(Am, b, np.zeros(A.n), L, U, search_max=M,
                                                           restart_max=RESTART_MAX, rtol=RTOL, tol_type=1)
            del L, U
            torch.cuda.synchronize()
            if it >= args.warmup:
                e2e_times.append(time.perf_counter() - t0)
        dropin.set_options()
        e2e_rel = true_rel(x)
        nf = nnzL + nnzU
        # A's values twice (both calls upload A), the factors up, b and x0 up;
        # the factors and x down
        h2d = 2 * (A.nnz * 8) + nf * 8 + 2 * A.n * 8
        d2h = nf * 8 + A.n * 8
        e2e = {"value": statistics.median(e2e_times), "unit": "s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "true_rel_resid": e2e_rel,
               "path": "data_PariLU_v0_3_prescribedSweeps + data_fgmres_householder_restart (fp32 factors)"}

    # ---- CPU baseline: oracle port (LACE's path restated in C, OpenMP), rank 0, N=1
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = cpu_baseline(A, b)

    # launches per solve: ParILU (4 initial-guess copies, the sweeps, 2 gathers,
    # the residual), 2 solve-plan value gathers, and per cycle the residual,
    # the first vector, m steps of [L solve, U solve, the one-kernel Arnoldi
    # step] (the step marks the next step's solve outputs, so the solves launch
    # no fills) and the x update (steps after convergence launch and exit at once)
    cycles = r_mixed.restarts + 1
    launches_per_solve = (4 + SWEEPS + 2 + 1) + 2 + cycles * (3 + M * 3)
    med = statistics.median(t_mixed)
    if world > 1:
        med = max_over_ranks(med)
    out = {
        "metric": METRIC,
        "value": med,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": med * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 factors+SpTRSV / fp64 FGMRES+SpMV",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": WORKLOAD, "precision": "mixed", "l2": "inputs larger than L2 (A 175 MB, "
                   "Krylov basis 0.86 GB)", "parallelism": "replicas" if world > 1 else "single"},
        "iterations": {"mixed": r_mixed.total_iterations, "fp64": r_fp64.total_iterations},
        "true_rel_resid": {"mixed": true_rel(x_mixed), "fp64": true_rel(x_fp64)},
        "fp64": {"value": statistics.median(t_fp64), "unit": "s"},
        "mgs": {"value": statistics.median(t_mgs), "unit": "s", "iterations": r_mgs.total_iterations,
                "true_rel_resid": true_rel(x_mgs),
                "path": "lace_gpu_fgmres_mgs (data_fgmres_restart semantics), fp32 factors"},
        "speedup_mixed_vs_fp64": statistics.median(t_fp64) / med,
        "kernels": {"sptrsv_pair_s": trsv_s, "sptrsv_pair_gbs": trsv_gbs, "sptrsv_pair_frac": trsv_gbs / hbm_peak,
                    "sptrsv_pair_algorithmic_bytes": ab["sptrsv_pair"], "sptrsv_pair_traffic": traffic_pair,
                    "sptrsv_schedule": sched, "spmv_s": spmv_s, "spmv_gbs": spmv_gbs,
                    "arnoldi_step_s": step_s},
        "roofline": {"bound": "hbm", "kernel": f"k_hh_step: one Arnoldi step (j = {STEP_J}, 16 basis columns; "
                     "operator, both dot-product sets, new reflector, next Krylov vector), mixed precision",
                     "achieved": step_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": step_gbs / hbm_peak,
                     "peak_source": peak_src + " (burst copy)", "algorithmic_bytes": sb,
                     "traffic": traffic,
                     "limiter": "FP64 pipe: (7 + 3(j+1)) FP64 FMAs per row, "
                                f"{(7 + 3 * (STEP_J + 1)) * A.n / step_s / 1e9:.0f} G FMA/s achieved against "
                                "595 G FMA/s measured with a plain FMA loop on this part"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": int(launches_per_solve * args.steps),
        "wall_s_timed": wall_mixed,
    }
    if rank == 0:
        print(json.dumps(out))
    ctx.close()


def cpu_baseline(A, b):
    """The oracle port on every host core: ParILU sweeps + FGMRES-Householder
    with exact FP64 triangular solves, one full solve (the bounded sample is
    the whole workload: it fits in tens of seconds)."""
    from oracle import oracle as orc
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    t0 = time.perf_counter()
    F = orc.parilu(A.row, A.col, A.val, SWEEPS, mode="sync")
    r = orc.fgmres({"kind": "csr", "row": A.row, "col": A.col, "val": A.val}, orc.ilu_precond(F), b,
                   search_max=M, restart_max=RESTART_MAX, rtol=RTOL)
    t = time.perf_counter() - t0
    return {"value": t, "unit": "s", "cores": cores, "kind": "port",
            "sample": f"one full solve ({r.total_iterations} FGMRES directions, FP64, exact sequential SpTRSV)",
            "converged": r.converged}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    A, b = build_problem()
    from oracle import oracle as orc
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    times = []
    r = None
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        F = orc.parilu(A.row, A.col, A.val, SWEEPS, mode="sync")
        r = orc.fgmres({"kind": "csr", "row": A.row, "col": A.col, "val": A.val}, orc.ilu_precond(F), b,
                       search_max=M, restart_max=RESTART_MAX, rtol=RTOL)
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    sample = f"one full solve per step ({r.total_iterations} FGMRES directions, FP64)"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": med, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": med * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": WORKLOAD, "precision": "fp64 (LACE's path is FP64)"},
        "cpu_baseline": {"value": med, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": med, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per launch of the dominant kernel (the Arnoldi step), if captured")
    ap.add_argument("--trsv-schedule", default=None,
                    help="R,chunks,warps,cluster: pin the sync-free solve schedule (the autotune's choice is "
                         "reported as roofline.schedule) - for profiling the same kernels under ncu, whose "
                         "launch overhead would change the autotune's choice")
    ap.add_argument("--only-mgs", action="store_true",
                    help="time only the FGMRES with modified Gram-Schmidt (for profiling its kernels)")
    ap.add_argument("--only-householder", action="store_true",
                    help="time only the FGMRES-Householder solve (for profiling its kernels)")
    ap.add_argument("--grid", type=int, default=GRID,
                    help="with --only-mgs / --only-householder: the convection-diffusion grid side "
                         "(a smaller case for ncu)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1 and args.impl == "ours":
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
