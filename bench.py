"""Benchmark: time to FP64 true relative residual 1e-8 on the 128^3
variable-coefficient problem (-div(k grad u), 7-point, k = exp(g), g a seeded
Gaussian random field, sigma 1, squared-exponential correlation length 8
cells) with two-level RAS (256 uneven box subdomains, overlap 1, one
piecewise-constant coarse vector per subdomain, FP64 coarse LU) inside
restarted GMRES(30).

One step = one complete solve from x0 = 0 of A x = b, b = A x*, x* ~ U[-1,1]
(seed 2), to ||b - A x||_2 / ||b||_2 <= 1e-8 checked in FP64.  Inputs
(matrix, factors, b) stay resident in HBM; the working set (matrix 217 MB
plus a 260-520 MB Krylov basis) is larger than the 129 MB L2, so no flush is
needed between steps.

  value : mixed-precision solver (FP32 sweeps over BF16 factors, FP32 inner
          Krylov basis, FP64 true residual / update / least squares / coarse
          LU), device-resident inputs, seconds per solve (CUDA events).
  e2e   : the same solve through the C ABI with host b and x (host<->device
          copies inside the timed region), host wall clock.
  fp64_gpu : the all-FP64 GPU solver on the same workload (the comparison
          the target ratio is quoted against).
  roofline : FP64 CSR SpMV of the operator, algorithmic bytes / kernel time.

`--impl reference` times the oracle (the CPU restatement of the reference's
OpenMP path, with the sparse restatement of its coarse space) on the same
workload with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

N_GRID = 128
NPARTS = 256
OVERLAP = 1
SPREAD = 0.08
RESTART = 30
RTOL = 1e-8
METRIC = "time_to_1e-8_fp64_true_residual"
WORKLOAD = ("varcoef3d_128^3_two_level_ras_256uneven_ov1_gmres30: -div(exp(g) grad u), "
            "sigma 1, corr 8 cells, n=2097152")


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def make_problem(sg, seed_offset=0):
    A = sg.make_varcoef_3d(N_GRID, N_GRID, N_GRID, 1.0, 8.0, seed=0 + seed_offset)
    part = sg.partition_boxes(N_GRID, N_GRID, N_GRID, NPARTS, SPREAD, seed=1)
    xs = sg.uniform(A.nrows, seed=2 + seed_offset)
    return A, part, xs


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<name>."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            m = re.match(r"\s*traffic_bytes_per_launch:\s*([0-9.eE+]+)", line)
            if m:
                return float(m.group(1))
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.device = device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- our arm
def run_ours(args):
    import torch

    import schwarz_gmres_dashboard_gb300 as sg

    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    ctx = sg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    # replicas: every rank solves its own instance (independent seeds)
    A, part, xs = make_problem(sg, seed_offset=rank)
    A.upload(ctx)
    n = A.nrows
    b = A.spmv(xs)
    bd = torch.from_numpy(b).to(f"cuda:{local}")
    xd = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")

    t0 = time.time()
    pc_mixed = sg.TwoLevelSchwarzPrecond(NPARTS, OVERLAP, sg.FineLevelType.RAS, part,
                                         factor_dtype=sg.BF16, sweep_dtype=sg.FP32, ctx=ctx)
    pc_mixed.setup(A)
    setup_mixed = time.time() - t0
    t0 = time.time()
    pc_fp64 = sg.TwoLevelSchwarzPrecond(NPARTS, OVERLAP, sg.FineLevelType.RAS, part, ctx=ctx)
    pc_fp64.setup(A)
    setup_fp64 = time.time() - t0
    p_mixed = sg.GMRESParams(restart=RESTART, max_iter=20000, tol=RTOL, tol_kind=sg.TOL_TRUE_REL,
                             precision=sg.FP32)
    p_fp64 = sg.GMRESParams(restart=RESTART, max_iter=20000, tol=RTOL, tol_kind=sg.TOL_TRUE_REL,
                            precision=sg.FP64)

    def device_solve(pc, prm):
        with torch.cuda.stream(stream):
            xd.zero_()
        return sg.gmres(A, bd, xd, pc, prm)

    def timed(pc, prm, steps, warmup):
        for _ in range(warmup):
            device_solve(pc, prm)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        results = []
        l0 = ctx.launch_count
        e0.record(stream)
        for _ in range(steps):
            results.append(device_solve(pc, prm))
        e1.record(stream)
        torch.cuda.synchronize()
        launches = ctx.launch_count - l0
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device=f"cuda:{local}")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms / steps, results, launches

    with Clocks(local) as clk:
        ms_mixed, res_mixed, launches = timed(pc_mixed, p_mixed, args.steps, args.warmup)
    x_mixed = xd.cpu().numpy()
    ms_fp64, res_fp64, _ = timed(pc_fp64, p_fp64, max(1, min(args.steps, 3)), 1)
    x_fp64 = xd.cpu().numpy()

    # e2e through the C ABI with host buffers (copies inside the timed region)
    bh = b.copy()
    e2e = []
    for i in range(args.warmup + args.steps):
        xh = np.zeros(n)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sg.gmres(A, bh, xh, pc_mixed, p_mixed)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e.append(t1 - t0)
    e2e_s = statistics.mean(e2e)

    # roofline: FP64 CSR SpMV of the operator
    nnz = A.nnz()
    spmv_bytes = nnz * (8 + 4) + 4 * (n + 1) + 2 * n * 8
    yd = torch.empty_like(bd)
    for _ in range(3):
        A.spmv(bd, yd)
    reps = 50
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(reps):
        A.spmv(bd, yd)
    s1.record(stream)
    torch.cuda.synchronize()
    spmv_s = s0.elapsed_time(s1) / 1e3 / reps
    peak, peak_kind = peaks()
    achieved = spmv_bytes / spmv_s / 1e9

    if rank != 0:
        return
    rm, rf = res_mixed[-1], res_fp64[-1]
    relerr_mixed_vs_fp64 = float(np.linalg.norm(x_mixed - x_fp64) / np.linalg.norm(x_fp64))
    relerr_vs_xstar = float(np.linalg.norm(x_mixed - xs) / np.linalg.norm(xs))

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline_sample(A, part, b, rf.iterations)

    line = {
        "metric": METRIC,
        "value": ms_mixed / 1e3,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32+bf16 inner / f64 outer",
        "data": "synthetic: seeded Gaussian random field coefficients, x* ~ U[-1,1]",
        "config": {
            "workload": WORKLOAD,
            "n": n, "nnz": nnz, "nparts": NPARTS, "overlap": OVERLAP, "restart": RESTART,
            "rtol": RTOL, "partition": f"boxes, seeded uneven cuts (spread {SPREAD})",
            "l2": "working set > L2 (no flush)",
            "solver": "GMRES(30) left-preconditioned, FP32 Krylov cycle from FP64 residual",
            "parallelism": f"replicas x{world}",
        },
        "iterations": rm.iterations,
        "cycles": rm.cycles,
        "true_rel_residual": rm.true_rel_residual,
        "rel_err_vs_fp64_gpu": relerr_mixed_vs_fp64,
        "rel_err_vs_xstar": relerr_vs_xstar,
        "solves_per_s": 1e3 / ms_mixed,
        "fp64_gpu": {"value": ms_fp64 / 1e3, "unit": "s", "iterations": rf.iterations,
                     "true_rel_residual": rf.true_rel_residual},
        "speedup_vs_fp64_gpu": ms_fp64 / ms_mixed,
        "setup_s": {"mixed": setup_mixed, "fp64": setup_fp64},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": 2 * n * 8,
                "d2h_bytes_per_step": n * 8},
        "roofline": {"kernel": "spmv_csr_fp64", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": profile_traffic("spmv_csr_fp64_varcoef128.md"),
                     "algorithmic_bytes": spmv_bytes, "kernel_us": spmv_s * 1e6},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))


def cpu_baseline_sample(A, part, b, iterations):
    """The oracle on one restart cycle (30 Arnoldi steps) of the same workload
    with all host threads; scaled to the FP64 GPU solver's iteration count."""
    try:
        from oracle.oracle import Oracle
        orc = Oracle()
        threads = os.cpu_count() or 1
        orc.set_threads(threads)
        pc = orc.precond("twolevel_ras", A, NPARTS, OVERLAP, part)
        t0 = time.perf_counter()
        orc.gmres(A, b, np.zeros(A.nrows), pc, restart=RESTART, max_iter=RESTART, tol=0.0)
        dt = time.perf_counter() - t0
        return {"value": dt / RESTART * iterations, "unit": "s", "cores": threads, "kind": "port",
                "sample": f"one GMRES(30) restart cycle (30 iterations) of the oracle two-level "
                          f"RAS solve, {dt:.2f} s, scaled to the {iterations} iterations the "
                          f"FP64 solver needs"}
    except Exception as e:  # the baseline is reported, never required
        return {"value": None, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                "sample": f"failed: {e}"}


# ---------------------------------------------------------------- reference arm
def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    import schwarz_gmres_dashboard_gb300 as sg  # host generators only
    from oracle.oracle import Oracle

    A, part, xs = make_problem(sg)
    orc = Oracle()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    b = orc.spmv(A, xs)
    bn = np.linalg.norm(b)
    pc = orc.precond("twolevel_ras", A, NPARTS, OVERLAP, part)
    # cycles of the oracle harness (GMRES(30), tol 0, warm start, FP64 true
    # residual checked between cycles); a step is one cycle
    x = np.zeros(A.nrows)
    cycle_times = []
    cycles_needed = None
    total = 0
    max_cycles = args.warmup + args.steps + 40
    while total < max_cycles:
        t0 = time.perf_counter()
        r = orc.gmres(A, b, x, pc, restart=RESTART, max_iter=RESTART, tol=0.0)
        dt = time.perf_counter() - t0
        x = r["x"]
        total += 1
        if total > args.warmup:
            cycle_times.append(dt)
        rel = np.linalg.norm(b - orc.spmv(A, x)) / bn
        if rel <= RTOL and cycles_needed is None:
            cycles_needed = total
        if cycles_needed is not None and len(cycle_times) >= args.steps:
            break
    sec_cycle = statistics.mean(cycle_times[: args.steps]) if cycle_times else float("nan")
    value = sec_cycle * (cycles_needed or total)
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec_cycle * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded Gaussian random field coefficients, x* ~ U[-1,1]",
        "config": {"workload": WORKLOAD, "n": A.nrows, "nnz": A.nnz()},
        "impl": "reference",
        "cycles_to_rtol": cycles_needed,
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                         "sample": f"{len(cycle_times[: args.steps])} timed GMRES(30) restart "
                                   f"cycles of the oracle (reference algorithm, OpenMP subdomain "
                                   f"loop, sparse restatement of the dense coarse space); value = "
                                   f"mean cycle time x {cycles_needed or total} cycles to 1e-8"},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=128,
                    help="grid edge (128 = the benchmark workload; smaller for profiling)")
    args = ap.parse_args()
    global N_GRID, NPARTS, WORKLOAD
    if args.grid != N_GRID:
        N_GRID = args.grid
        NPARTS = max(8, min(NPARTS, round(256 * (args.grid / 128) ** 3)))
        WORKLOAD = WORKLOAD.replace("128^3", f"{N_GRID}^3").replace("256uneven", f"{NPARTS}uneven")
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
