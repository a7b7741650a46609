"""Benchmark of the nonlocal-density Newton path on one GB300.

Workload (configuration 2): 3-D FMT1 + WCA Lennard-Jones fluid
(eps=1, r_c=2.5 sigma, kT*=1.2), sigma=1, 128^3 nodes at dx=0.1 sigma,
rho_b=0.6, periodic in y and z, a rough 12-3 LJ wall (eps_w=1, 16x16 patches
of U(-0.5,0.5) sigma heights, seeded) on the low-x side, bulk on the high-x side.

A step is one Newton solve from the initial state (rho_b exp(-V) with its own
weighted densities) to ||R||_2 <= 1e-8: residual fills (FP32 stencil sums while
||R||_2 > 0.1, FP64-accurate after: the attraction sum as an FP64 FFT
convolution, the short stencils as float-float sums), Schur-complement GMRES
whose products take the 3-D attraction sum as an FP32 FFT convolution or on
the tensor cores (tcgen05, split FP16 x3), whichever the handle timed faster,
and the other stencils in FP32 (inexact Newton, Eisenstat-Walker tolerances),
and the damped update.  The value is Newton iterations per second over the K
timed solves.  Beside it: the plain FP64 path (every sum FP64-accurate in fills
and products, the long ones as FP64 FFT convolutions, same driver and target)
timed over a whole solve, and continued to ||R||_2 <= 1e-10 as the reference
solution for the mixed solution's maximum density error; and one iteration
with direct FP64 sums.  The inputs (12 unknowns x 128^3 doubles = 201 MB, plus
the 200+ MB of padded fields) exceed the 129 MB L2, so no explicit flush is
done between steps.

`--impl reference` times the reference's fill algorithm (the C oracle under
oracle/, a restatement of the reference's fill, on the reference's own stencil
tables and bulk constants) on the host cores on a bounded sample of the same
workload and prints the same metric with its cost model.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("Newton iterations/s of a mixed-precision solve to ||R||_2 <= 1e-8, 128^3 FMT1+WCA "
          "(FP32-class stencil sums in the Schur products, FP64 residual)")
UNIT = "Newton iter/s"
WORKLOADS = {
    "config2": "config2: 3-D FMT1+WCA, 128^3, dx=0.1, rho_b=0.6, rough 12-3 LJ wall, periodic y,z",
    "config4": ("config4: 3-D FMT1+WCA, 256^3, dx=0.08, rough 12-3 LJ wall, periodic y,z; rho_b 0.70 by continuation "
                "0.60 -> 0.65 -> 0.70 (the rho_b=0.75 of the specification has no solution this model reaches: "
                "the contact peak grows without bound past rho_b ~ 0.705)"),
    "config5": ("config5: 64 slit pores, FMT1+WCA, 32 1-D (dx=0.01, widths U(3,40)) and 32 2-D (n^2, "
                "n in [100,400], dx=0.05, patterned walls), rho_b U(0.05,0.8) each; seed 2024"),
}


def make_problem(args):
    from tramonto_gb300 import setup
    if args.workload == "config4":
        return setup.config4()
    return setup.config2(n=args.n)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=128, help="grid of the config2 workload")
    ap.add_argument("--workload", default="config2", choices=["config2", "config4", "config5"])
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="Newton iterations timed with direct FP64 stencil sums (0: skip)")
    ap.add_argument("--lin-tol", type=float, default=1e-6)
    ap.add_argument("--lin-maxit", type=int, default=200)
    ap.add_argument("--resid-tol", type=float, default=1e-8)
    ap.add_argument("--max-newton", type=int, default=40)
    ap.add_argument("--switch", type=float, default=0.1)
    ap.add_argument("--cpu-sample-planes", type=int, default=0,
                    help="z-planes of the CPU sample (0: 2 for the GPU arm's one-core baseline, a quarter of the host "
                         "threads for the reference arm)")
    ap.add_argument("--k-gmres", type=float, default=7.43,
                    help="GMRES iterations per Newton iteration for the reference arm's cost model (the GPU arm "
                         "prints its own as gmres_iters_per_newton_iter)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fft32-policy", type=int, default=-1, choices=[-1, 0, 1],
                    help="FP32 sums as FP32 FFT convolutions: -1 chosen by timing each sum's first use (default), "
                         "1 always, 0 never (profiler runs fix the choice, since their timings are not the real ones)")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 solve and the density error (launch lists and profiles)")
    ap.add_argument("--light", action="store_true",
                    help="one repetition of each FP64 kernel-family timing (large workloads)")
    ap.add_argument("--products", default="fp16tc", choices=["fp16tc", "fp32"],
                    help="arithmetic of the Schur products' attraction sums")
    ap.add_argument("--accurate-fill", default="fft", choices=["ff", "fft", "fp64"],
                    help="arithmetic of the fills once ||R||_2 < switch: float-float sums, FP64 FFT sums or "
                         "direct FP64 sums")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# dram__bytes_read.sum + dram__bytes_write.sum of one k_sten_tc launch at 128^3 (ncu, one launch)
TC_TRAFFIC_BYTES = 47.724e6 + 0.538e6
# DRAM bytes per algorithmic byte of the FP32 y/z FFT pass launches (k_fft_stridedw<float2>) of a timed solve at
# 128^3: ncu dram__bytes_read.sum + dram__bytes_write.sum summed over the launches, divided by their algorithmic
# bytes (ncu flushes the caches before each profiled launch, so every launch reads from DRAM there)
FFT32_PASS_TRAFFIC_BYTES_PER_BYTE = (27604.527e6 + 3098.825e6) / (512 * 99.893e6)


def tc_issued_flops(p):
    """MMA flops the tensor-core attraction sum issues per launch: per stencil line (oy, oz) and output
    tile (64 x by 128 y of one z-plane), 3 MMAs of 128x64x16 per 16-input K-step of the line's band."""
    from tramonto_gb300.problem import UATT
    off = p.stencils[(UATT, 0)][0]
    lines = {}
    for ox, oy, oz in off:
        lines[(oz, oy)] = max(lines.get((oz, oy), 0), abs(int(ox)))
    ksteps = sum((32 + 63 + l) // 16 - (32 - l) // 16 + 1 for l in lines.values())
    tiles = -(-p.nx[0] // 64) * -(-p.nx[1] // 128) * p.nx[2]
    return float(tiles) * ksteps * 3 * 2 * 128 * 64 * 16


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def conv_flops_per_apply(p):
    """Logical flops of the stencil sums of one Schur product (2 per multiply-add)."""
    nd = p.ndim
    fwd = tr = att = 0
    for c in range(p.ncomp):
        Lt = len(p.stencils[(1, c)][1])
        Ld = len(p.stencils[(0, c)][1])
        nout = (1 + nd) if p.single_size else (3 + 2 * nd)
        fwd += Lt + nout * Ld
        tr += Lt + (1 + nd) * Ld
    if p.attraction:
        for k in range(p.ncomp * p.ncomp):
            att += len(p.stencils[(2, k)][1])
    return 2.0 * p.nnodes * (fwd + tr + att), 2.0 * p.nnodes * att


def cpu_baseline(p, x, k_gmres, planes, threads=1):
    """Time the C oracle's residual fill on `planes` x-planes of the workload and
    extrapolate to one Newton iteration = (1 + k) fills (k = GMRES iterations)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    o = orc.Oracle(p)
    nxy = p.nx[0] * p.nx[1]
    # sample: the first `planes` z-planes (full x-y extent, wall and bulk included)
    t0 = time.perf_counter()
    if threads <= 1:
        o.resid_rows(x, 0, planes * nxy)
        dt = time.perf_counter() - t0
        nodes = planes * nxy
    else:
        from concurrent.futures import ThreadPoolExecutor
        # ctypes releases the GIL: one row range per thread
        per = max(1, planes // threads)
        ranges = [(i * per * nxy, (i + 1) * per * nxy) for i in range(threads)]
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda r: o.resid_rows(x, r[0], r[1]), ranges))
        dt = time.perf_counter() - t0
        nodes = per * threads * nxy
    t_fill = dt * p.nnodes / nodes
    t_iter = (1 + k_gmres) * t_fill
    return {"value": 1.0 / t_iter, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle residual fill of {nodes} of {p.nnodes} nodes ({dt:.1f} s); Newton iteration "
                      f"extrapolated as (1 + {k_gmres:.0f} GMRES iterations) x full fill",
            "t_fill_s": t_fill}


def workload_config(args, ladder=None):
    """The `config` dict of both arms' JSON lines (the same dict, built from the command line alone)."""
    if args.workload == "config4":
        grid, dx, rho_b = [256] * 3, 0.08, 0.7
    else:
        grid, dx, rho_b = [args.n] * 3, 0.1, 0.6
    return {"workload": WORKLOADS[args.workload],
            "step": (f"the continuation {ladder}, each rung solved to ||R||_2 <= {args.resid_tol:g}" if ladder
                     else f"one Newton solve from the initial state to ||R||_2 <= {args.resid_tol:g}"),
            "grid": grid, "dx": dx, "seed": 1234, "rho_b": rho_b, "continuation": ladder, "kT": 1.2, "rcut": 2.5,
            "lin_tol_floor": args.lin_tol, "fp32_until_resid": args.switch, "inputs_exceed_l2": True,
            "l2_flush": "none (working set > L2)"}


def run_reference(args):
    """Reference arm: the reference's fill algorithm (the C oracle, a restatement of it) on all host cores.

    Nothing from the product package is imported: the problem comes from oracle/workload.py (the reference's own
    stencil tables and bulk constants, the workload's seeded wall field).  Each step is one residual fill of a
    sample of z-planes of the 128^3 grid at the state the GPU arm's solves start from (densities and their own
    weighted densities and mean field); ms_per_step is its measured time.  The Newton-iteration rate is the
    cost model of the reference's own CPU path: (1 + k) fills per Newton iteration (the assembled Jacobian of
    the 128^3 problem holds ~1e11 entries, so its GMRES cannot run here), k = the GPU arm's GMRES iterations per
    Newton iteration (--k-gmres), the full fill = the sample's time scaled by the node count."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload != "config2":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm times the 128^3 workload only"}))
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    import workload
    p = workload.config2_problem(args.n)
    o = orc.Oracle(p)
    threads = os.cpu_count() or 1
    planes = args.cpu_sample_planes if args.cpu_sample_planes > 0 else max(2, threads // 4)
    t0 = time.perf_counter()
    x = workload.initial_state(p, o, planes, threads)
    t_state = time.perf_counter() - t0
    ranges = workload.plane_ranges(p, range(planes), threads)
    nodes = sum(e - b for b, e in ranges)

    def step():
        from concurrent.futures import ThreadPoolExecutor
        t = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda r: o.resid_rows(x, r[0], r[1]), ranges))
        return time.perf_counter() - t

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(max(1, args.steps))]
    t_sample = float(np.median(times))
    t_fill = t_sample * p.nnodes / nodes
    k = args.k_gmres
    v = 1.0 / ((1.0 + k) * t_fill)
    sample = (f"oracle residual fill of {planes} z-planes ({nodes} of {p.nnodes} nodes) on {threads} threads, "
              f"median {t_sample:.2f} s per step; Newton iteration = (1 + k) full fills, k = {k:g}")
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_sample * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(args),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "model": {"step": "one residual fill of the sampled z-planes (ms_per_step is its measured time)",
                     "sample_fraction": nodes / p.nnodes, "full_fill_s": t_fill,
                     "newton_iteration": "(1 + k) full fills", "k": k,
                     "k_source": "GMRES iterations per Newton iteration of the GPU arm's solve "
                                 "(its gmres_iters_per_newton_iter), passed as --k-gmres",
                     "state_setup_s": t_state,
                     "inputs": "stencil tables and bulk constants from the reference's own set-up "
                               "(tests/golden/sten3d_dx010.npz), seeded wall field"}}
    print(json.dumps(out))


def run_config5(args):
    """Configuration 5: every slit-pore problem solved at its state point from its initial state, with
    dN/d(beta mu) by the adjoint, in mixed precision and in plain FP64; wall time of the whole sweep
    (set-up, solve and derivative of each problem) and Newton iterations per second."""
    import torch
    import torch.distributed as dist
    from tramonto_gb300 import isotherm, ranks, setup
    world, rank, local = ranks.env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    specs = ranks.shard(setup.config5(), rank, world)   # independent problems dealt out to the ranks
    isotherm.sweep(specs[:2], mixed=True)               # warm-up (library load, first contexts)
    out = {}
    for name, mixed in (("mixed", True), ("fp64", False)):
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        recs = isotherm.sweep(specs, mixed=mixed)
        wall = time.perf_counter() - t0
        iters, wall, rate = ranks.whole_job_rate(sum(r["iters"] for r in recs), wall * 1e3, device="cuda")
        wall *= 1e-3
        out[name] = {"wall_s": wall, "newton_iters": int(iters),
                     "converged": int(ranks.reduce_sum(sum(r["converged"] for r in recs), "cuda")),
                     "iters_per_s": rate, "wall_s_1d_rank0": sum(r["wall_s"] for r in recs if r["ndim"] == 1),
                     "wall_s_2d_rank0": sum(r["wall_s"] for r in recs if r["ndim"] == 2)}
        if mixed:
            out["dN_dbetamu_sample"] = [(r["ndim"], r["nodes"], round(r["rho_b"], 4), r.get("dN_dbetamu"))
                                        for r in recs[::8]]
    if rank != 0:
        dist.destroy_process_group()
        return
    line = {"metric": "Newton iterations/s over the configuration-5 slit-pore sweep (mixed precision)",
            "value": out["mixed"]["iters_per_s"], "unit": "Newton iter/s", "n_gpus": world, "steps": 1, "warmup": 1,
            "ms_per_step": out["mixed"]["wall_s"] * 1e3, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f64 residual near the solution, f32 stencil sums in the Schur products",
            "data": "synthetic", "config": {"workload": WORKLOADS["config5"], "step": "the whole sweep"},
            "sweep": out, "speedup_mixed_vs_fp64_wall": out["fp64"]["wall_s"] / out["mixed"]["wall_s"]}
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "config5":
        run_config5(args)
        return
    import torch
    import torch.distributed as dist
    from tramonto_gb300 import ranks
    world, rank, local = ranks.env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from tramonto_gb300 import native, setup
    from tramonto_gb300.problem import DELTA, THETA, UATT
    t_setup = t_start = time.perf_counter()
    p, meta = make_problem(args)
    prod_prec = native.FP16TC if args.products == "fp16tc" else native.FP32
    s = native.Solver(p, device=local, precision=native.FP32)
    stream = torch.cuda.current_stream()
    s.set_stream(stream.cuda_stream)
    x0 = setup.initial_state(s, p, max_enhancement=meta.get("initial_cap"))
    t_setup = time.perf_counter() - t_setup
    n = p.nunk * p.nnodes
    x0_dev = torch.from_numpy(x0).to("cuda").contiguous()
    dx = torch.empty_like(x0_dev)

    fill_mode = {"ff": native.FILL_MIXED_FF, "fft": native.FILL_MIXED_FFT, "fp64": native.FILL_MIXED}[args.accurate_fill]

    def mixed_mode():
        s.set_precision(prod_prec)
        s.set_fill_arithmetic(fill_mode, switch_norm=args.switch)

    if args.fft32_policy != -1:
        s.set_fft32_policy(args.fft32_policy)

    ladder = meta.get("ladder")

    def solve(xt=dx, resid_tol=None, lin_tol=None):
        """One step: a Newton solve from the initial state, or the continuation along the workload's ladder of
        bulk densities (each rung warm-started from the previous solution); totals over the rungs."""
        xt.copy_(x0_dev)
        kw = dict(resid_tol=resid_tol or args.resid_tol, max_iter=args.max_newton, lin_tol=lin_tol or args.lin_tol,
                  lin_max_iter=args.lin_maxit, allow_noconv=True)
        if not ladder:
            return s.newton_solve_device(xt, **kw)
        it_t = li_t = 0
        rn = float("inf")
        for rb in ladder:
            s.set_bulk([rb])
            it, rn, li = s.newton_solve_device(xt, **kw)
            it_t += it
            li_t += li
        return it_t, rn, li_t

    def progress(msg):
        if rank == 0:
            print(f"[bench {time.perf_counter() - t_start:8.1f} s] {msg}", file=sys.stderr, flush=True)

    progress(f"set-up done ({p.nnodes} nodes, {p.nunk} unknowns per node)")
    mixed_mode()
    for w in range(args.warmup):
        it_w, rn_w, li_w = solve()
        torch.cuda.synchronize()
        progress(f"warm-up solve {w}: {it_w} Newton iterations, {li_w} GMRES, ||R||_2 = {rn_w:.2e}")
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    s.reset_stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters = lin_iters = 0
    final_r = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed_solves")   # the launch list's window (ncu --nvtx-include timed_solves/)
        e0.record(stream)
        for _ in range(args.steps):
            it, rn, li = solve()
            iters += it
            lin_iters += li
            final_r.append(rn)
            progress(f"timed solve: {it} Newton iterations, {li} GMRES, ||R||_2 = {rn:.2e}")
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    st = s.stats()
    # the roofline kernel in one more solve, the same as a timed one: a CUDA event pair on the solver's stream around
    # every FP32 y/z FFT pass launch gives its average launch duration and algorithmic bytes per launch
    s.pass_timer_begin()
    solve(torch.empty_like(dx))
    torch.cuda.synchronize()
    pt_launches, pt_ms, pt_bytes, pt_transforms = s.pass_timer_end()
    choices = {name: s.fft32_choice(t, 0) for name, t in (("theta", THETA), ("delta", DELTA), ("attraction", UATT))}
    ms_total = e0.elapsed_time(e1)
    # one replica per rank: Newton iterations of all ranks over the slowest rank's time
    _, ms_total, value = ranks.whole_job_rate(max(1, iters), ms_total, device="cuda")
    ms_per_solve = ms_total / args.steps
    ms_per_iter = ms_total / max(1, iters)
    x_mixed = dx.clone()
    # the returned state's residual re-evaluated with FP64 sums
    s.set_fill_arithmetic(native.FILL_FP64)
    R_chk = torch.empty_like(dx)
    s.fill_device(x_mixed, R_chk, 1)
    resid_fp64 = float(torch.linalg.vector_norm(R_chk).item())
    del R_chk
    progress(f"residual of the solution in FP64: {resid_fp64:.2e}")

    # kernel-family timings at the converged state
    R = torch.empty_like(dx)
    s.set_fill_arithmetic(native.FILL_FP64)
    v2 = torch.randn(p.ncomp * p.nnodes, dtype=torch.float64, device="cuda")
    y2 = torch.empty_like(v2)

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    rep64 = 1 if args.light else 3
    t_fill = timed(lambda: s.fill_device(x_mixed, R, 0), reps=rep64)
    s.set_fill_arithmetic(native.FILL_FF)
    t_fill_ff = timed(lambda: s.fill_device(x_mixed, R, 0), reps=rep64)
    s.set_fill_arithmetic(native.FILL_FFT)
    t_fill_fft = timed(lambda: s.fill_device(x_mixed, R, 0), reps=3)
    s.set_fill_arithmetic(native.FILL_FP32)
    t_fill32 = timed(lambda: s.fill_device(x_mixed, R, 0))
    s.set_precision(native.FP32)
    t_apply32 = timed(lambda: s.schur_device(v2, y2), reps=5)
    s.set_precision(native.FP16TC)
    t_apply_tc = timed(lambda: s.schur_device(v2, y2), reps=5)
    s.set_precision(native.FP64)
    t_apply64 = timed(lambda: s.schur_device(v2, y2), reps=1 if args.light else 2)
    progress("kernel-family timings done")
    # dominant kernel of the Schur products: the attraction (WCA) stencil sum
    t_wca_tc = s.time_stencil_sum(UATT, 0, native.FP16TC, reps=5)
    t_wca32 = s.time_stencil_sum(UATT, 0, native.FP32, reps=5)
    t_wca64 = s.time_stencil_sum(UATT, 0, native.FP64, reps=1)
    t_wca_ff = s.time_stencil_sum(UATT, 0, native.FILL_FF, reps=rep64)
    t_wca_fft = s.time_stencil_sum(UATT, 0, native.FILL_FFT, reps=3)
    t_wca_fft32 = s.time_stencil_sum(UATT, 0, native.TIME_FFT32, reps=5)
    L_att = len(p.stencils[(UATT, 0)][1])
    flops_att = 2.0 * p.nnodes * L_att
    mma_flops = tc_issued_flops(p)
    # The plain FP64 path: every sum FP64-accurate in the fills and in the Schur products (the long 3-D sums as
    # FP64 FFT convolutions, the short ones in float-float arithmetic), the same Newton driver and target, timed
    # over a whole solve; then continued to ||R||_2 <= 1e-10 with tight linear solves as the FP64 solution the
    # mixed solution's density is compared with.
    fp64_ms = it64 = li64 = rn64 = dens_err = dens_max = None
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if not args.no_plain:
        s.set_precision(native.FP64_FFT)
        s.set_fill_arithmetic(native.FILL_FFT)
        x64 = torch.empty_like(dx)
        torch.cuda.synchronize()
        a.record(stream)
        it64, rn64, li64 = solve(x64)
        b.record(stream)
        torch.cuda.synchronize()
        fp64_ms = a.elapsed_time(b) / max(1, it64)
        progress(f"plain FP64 solve: {it64} Newton iterations, {li64} GMRES, {fp64_ms:.1f} ms per iteration")
        s.newton_solve_device(x64, resid_tol=1e-10, max_iter=args.max_newton, lin_tol=1e-10, lin_max_iter=args.lin_maxit,
                              allow_noconv=True)
        rho = slice(p.first_rho, p.first_rho + p.ncomp)
        dens_err = float((x_mixed[rho] - x64[rho]).abs().max().item())
        dens_max = float(x64[rho].abs().max().item())
        progress(f"max |rho_mixed - rho_fp64| = {dens_err:.2e} (max rho {dens_max:.3f})")
        del x64
    # the same iteration with direct FP64 stencil sums (no FFT, no float-float) in fills and products
    s.set_precision(native.FP64)
    s.set_fill_arithmetic(native.FILL_FP64)
    direct_ms = None
    if args.fp64_steps > 0:
        dxd = x0_dev.clone()
        s.newton_device(dxd, max_iter=1, lin_tol=args.lin_tol, lin_max_iter=args.lin_maxit, allow_noconv=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(args.fp64_steps):
            s.newton_device(dxd, max_iter=1, lin_tol=args.lin_tol, lin_max_iter=args.lin_maxit, allow_noconv=True)
        b.record(stream)
        torch.cuda.synchronize()
        direct_ms = a.elapsed_time(b) / args.fp64_steps
        del dxd
    # end to end through the C ABI with host buffers: copies of the state in and out inside the timed region
    mixed_mode()
    xh = torch.from_numpy(x0.copy()).pin_memory().numpy()   # the caller's state in pinned host memory
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it_e2e = 0
    for rb in (ladder or [None]):
        if rb is not None:
            s.set_bulk([rb])
        xh, it_k, rn_e2e, _ = s.newton_solve(xh, resid_tol=args.resid_tol, max_iter=args.max_newton,
                                             lin_tol=args.lin_tol, lin_max_iter=args.lin_maxit, allow_noconv=True,
                                             inplace=True)
        it_e2e += it_k
    e2e_s = time.perf_counter() - t0
    hbm, bf16, peak_src = peaks()
    t_dom = t_wca_tc if args.products == "fp16tc" else t_wca32
    # the launch list's leading kernel: one y or z pass of the FP32 FFT sums over the half spectrum
    t_pass_y, nh, nr = s.time_fft_pass(native.FP32, 1, reps=20)
    t_pass_z, _, _ = s.time_fft_pass(native.FP32, 2, reps=20)
    t_pass = 0.5 * (t_pass_y + t_pass_z)
    pass_bytes = 2.0 * nh * 8.0                          # the half spectrum (complex FP32) read and written
    pt_launches = max(1, pt_launches)
    launch_ms, launch_bytes = pt_ms / pt_launches, pt_bytes / pt_launches
    launch_gbs = launch_bytes / (launch_ms * 1e-3) / 1e9
    t_pass64, _, _ = s.time_fft_pass(native.FP64, 1, reps=10)
    fft_flops = 2 * 2.5 * nr * math.log2(nr) + 6.0 * nh  # two real transforms and the spectral product
    ach_tf = flops_att / (t_dom * 1e-3) / 1e12
    issued_tf = mma_flops / (t_wca_tc * 1e-3) / 1e12
    if rank == 0:
        cb = None
        if not args.no_cpu_baseline:
            k = max(1.0, lin_iters / max(1, iters))
            cb = cpu_baseline(p, x_mixed.cpu().numpy(), k, planes=args.cpu_sample_planes or 2, threads=1)
            cb.pop("t_fill_s", None)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_solve, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ({"ff": "f64-accurate residual near the solution (float-float 3-D sums, rechecked in f64)",
                       "fft": "f64 residual near the solution (3-D sums as f64 FFT convolutions, rechecked by the "
                              "direct f64 sums)",
                       "fp64": "f64 residual near the solution"}[args.accurate_fill] +
                      ("; Schur products: attraction sums as f32 FFT convolutions or split-f16 x3 tensor-core sums, "
                       "whichever the handle timed faster (roofline.ms_per_launch against "
                       "roofline.tensor_core_kernel), f32 other stencil sums"
                       if args.products == "fp16tc" else
                       "; Schur products: attraction sums as f32 FFT convolutions or f32 slab sums, whichever is "
                       "faster, f32 other stencil sums")),
            "data": "synthetic",
            "config": workload_config(args, ladder),
            "newton_iters_per_step": iters / args.steps, "ms_per_newton_iter": ms_per_iter,
            "gmres_iters_per_newton_iter": lin_iters / max(1, iters), "final_resid_norm2": max(final_r),
            "final_resid_norm2_fp64_recheck": resid_fp64, "accurate_fill": args.accurate_fill,
            "gpu_launches": int(st["kernel_launches"]),
            "fp32_sum_choices": choices,
            "clocks": clk.summary(),
            "e2e": {"value": it_e2e / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * 8 * len(ladder or [0]),
                    "d2h_bytes_per_step": n * 8 * len(ladder or [0]),
                    "final_resid_norm2": rn_e2e},
            # the largest share of the timed solve's launch list: the y and z passes of the FP32 FFT stencil sums
            # (every stencil sum of the Schur products and FP32 fills), each reading and writing the half spectrum
            "roofline": {"bound": "hbm",
                         "kernel": "k_fft_stridedw<float2>: the y and z passes of the FP32 FFT stencil sums (one warp "
                                   "per line, 16 lines per CTA), each launch a batch of transforms over the half "
                                   "spectrum",
                         "achieved": launch_gbs, "peak": hbm, "unit": "GB/s", "frac": launch_gbs / hbm,
                         "peak_source": f"{peak_src} HBM copy (burst)",
                         "measured": f"CUDA events around each of the {pt_launches} launches of one solve like the "
                                     "timed ones",
                         "ms_per_launch": launch_ms, "launches_per_solve": pt_launches,
                         "transforms_per_launch": pt_transforms / pt_launches,
                         "algorithmic": f"{launch_bytes / 1e6:.1f} MB per launch on average: per transform the "
                                        f"{nh}-point complex FP32 half spectrum ({nh * 8 / 1e6:.1f} MB) written once "
                                        "and read once, or the two operands of each spectral product read",
                         "traffic": (FFT32_PASS_TRAFFIC_BYTES_PER_BYTE * launch_bytes
                                     if args.workload == "config2" and args.n == 128 else None),
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum over the launches of a "
                                           "timed solve at 128^3, per algorithmic byte, times this launch average",
                         "single_transform_pass": {"ms_y": t_pass_y, "ms_z": t_pass_z,
                                                   "achieved_gbs": pass_bytes / (t_pass * 1e-3) / 1e9,
                                                   "note": "one transform per launch, 768 CTAs: 1.26 waves"},
                         "fp64_pass_ms_per_launch": t_pass64,
                         "fft32_attraction_sum": {
                             "ms_per_sum": t_wca_fft32,
                             "fft_flops": fft_flops,
                             "fft_tflops": (fft_flops / (t_wca_fft32 * 1e-3) / 1e12) if fft_flops else None,
                             "counted": "2 x 2.5 NR log2 NR for the real forward and inverse transforms of the "
                                        f"{nr}-point box, 6 per half-spectrum point for the product",
                             "logical_tflops": flops_att / (t_wca_fft32 * 1e-3) / 1e12,
                             "logical": f"2 x {L_att} stencil points x {p.nnodes} nodes per sum"},
                         "tensor_core_kernel": {
                             "kernel": "k_sten_tc (tcgen05 split FP16 x3), the direct sum it replaces",
                             "ms_per_launch": t_wca_tc, "bound": "tensor", "achieved_logical_tflops": ach_tf,
                             "peak": bf16, "frac": ach_tf / bf16, "issued_mma_tflops": issued_tf,
                             "issued_mma_frac": issued_tf / bf16,
                             "traffic": (TC_TRAFFIC_BYTES if args.workload == "config2" and args.n == 128 else None),
                             "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at "
                                               "128^3"},
                         "fp32_slab_ms_per_launch": t_wca32, "fp32_slab_tflops": flops_att / (t_wca32 * 1e-3) / 1e12,
                         "fp64_ms_per_launch": t_wca64},
            # the attraction sum of the accurate fills: an FP64 FFT convolution by default (--accurate-fill fft;
            # its cost is two real transforms of the 180 x 128 x 128 box, independent of the stencil's length),
            # else the float-float sum, bound by the FP32 issue rate (12 FP32 operations per term; nominal 152 SMs
            # x 128 lanes x clock), reported here for comparison
            "fill_attraction_sum": {"fft_ms_per_sum": t_wca_fft,
                                    "fft_logical_tflops": flops_att / (t_wca_fft * 1e-3) / 1e12,
                                    "fft_vs_float_float": t_wca_ff / t_wca_fft},
            "float_float_attraction_sum": {"kernel": "k_conv_slab_ff (float-float attraction sum, --accurate-fill ff)",
                            "bound": "fp32 issue", "ms_per_launch": t_wca_ff,
                            "achieved": 12.0 * flops_att / 2.0 / (t_wca_ff * 1e-3) / 1e12,
                            "peak": 152 * 128 * (clk.summary().get("sm_max_mhz") or 2070.0) * 1e6 / 1e12,
                            "unit": "Top/s (FP32 operations)",
                            "frac": (12.0 * flops_att / 2.0 / (t_wca_ff * 1e-3)) /
                                    (152 * 128 * (clk.summary().get("sm_max_mhz") or 2070.0) * 1e6),
                            "peak_source": "nominal FP32 issue rate at the maximum SM clock",
                            "logical_tflops": flops_att / (t_wca_ff * 1e-3) / 1e12},
            "cpu_baseline": cb,
            "breakdown_ms": {"fill_fp64": t_fill, "fill_float_float": t_fill_ff, "fill_fft": t_fill_fft,
                             "attraction_sum_fft": t_wca_fft, "fill_fp32": t_fill32,
                             "schur_apply_fp32": t_apply32,
                             "schur_apply_fp16tc": t_apply_tc,
                             "schur_apply_fp64": t_apply64, "schur_applies_in_timed_steps": int(st["schur_applies"])},
            "plain_fp64": None if fp64_ms is None else {
                "ms_per_newton_iter": fp64_ms, "newton_iters": it64, "gmres_iters": li64, "final_resid_norm2": rn64,
                "arithmetic": "FP64-accurate fills and Schur products: 3-D stencil sums as FP64 FFT convolutions "
                              "where the cost model finds them cheaper than float-float direct sums",
                "speedup_mixed_vs_fp64_per_iter": fp64_ms / ms_per_iter,
                "speedup_mixed_vs_fp64_per_solve": (fp64_ms * it64) / ms_per_solve},
            "plain_fp64_direct_sums": {"ms_per_newton_iter": direct_ms,
                                       "speedup_mixed_vs_direct_per_iter": (direct_ms / ms_per_iter)
                                       if direct_ms else None},
            "max_density_err_vs_fp64": dens_err,
            "density_err_reference": None if dens_max is None else
                ("the FP64 path's solution continued to ||R||_2 <= 1e-10 (linear tolerance 1e-10); max density "
                 f"{dens_max:.4f}"),
            "setup_s": t_setup,
        }
        print(json.dumps(out))
    s.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
