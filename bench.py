#!/usr/bin/env python
"""Benchmark of the immersed-boundary fractional step on GB300.

Workload: flow past a sphere, 192x128x128 cells (3,145,728 interior cells),
body-clustered grid on [-5,15]x[-5,5]^2, 20480-triangle icosphere r = 0.5,
Re 300, dt 5e-3, uniform inflow, pressure outlet, free-slip sides; the
pressure solve runs to max|div U^{n+1}| <= 1e-8 on fluid cells every step,
momentum to the reference drivers' relative tolerance 1e-6.  Synthetic,
seeded inputs (the reference has no public dataset).

Metric: Mcell-steps/s = interior cells x steps / seconds, for the
mixed-precision step (the autotuner's choice among the mixed forms; on this
workload IBM3D_MIXED32: FP32 explicit stages and momentum solve, the
pressure BiCGSTAB on double-float vectors with the FP32 multigrid, FP64
right-hand side, solution, scalars and divergence check), with the plain
FP64 step measured beside it on the same state ("fp64", "mixed_vs_fp64")
and the velocity difference between the two after the run
("error_vs_fp64").
  value : device time (CUDA events on the solver's stream) of K steps with
          the state resident in HBM (the step's working set, >1 GB, is far
          larger than the 129 MB L2).  Each step is one recorded CUDA graph.
  e2e   : the same K steps through the C ABI with HOST buffers: every step
          uploads u1, u2, u3, p from pinned host memory
          (IBMSolver_init_flow_array), runs IBMSolver_iterate(1) and reads
          the four fields back (IBMSolver_get_field); host wall clock.
  roofline: the dominant kernel (fine-grid colour pass of the pressure
          multigrid) timed with CUDA events on the solver's stream, against
          the measured HBM copy bandwidth.
Default run: N=1, K=10 timed steps after W=3 warm-up steps;
--precision fp64 makes the plain FP64 step the headline.

--impl reference runs the CPU restatement of the reference time step
(oracle/, OpenMP on every host core) on the same workload and metric.
Under torchrun (N>1) every rank advances its own replica of the case (the
single-case path does not shard); value is the total over ranks divided by
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import importlib
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

DIV_TOL = 1e-8
MOM_TOL = 1e-6


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _barrier_max(value, world):
    """Barrier + max over ranks (gloo; the path has no data collective)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        dist.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                t = [x.strip() for x in line.split(",")]
                if len(t) >= 9:
                    rows.append(t)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_launch(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/roofline_traffic.txt: '<kernel> <workload> <bytes>'), or None."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    try:
        for line in open(path):
            t = line.split()
            if len(t) >= 3 and not line.startswith("#") and t[0] == kernel:
                return float(t[2])
    except OSError:
        pass
    return None


def oracle_case(case, lvset, threads, div_tol=DIV_TOL, tol=MOM_TOL):
    c = {k: v for k, v in case.items() if k not in ("stl", "init", "name")}
    c.update(lvset=lvset, threads=threads, div_tol=div_tol, tol=tol)
    return c


def cpu_level_set(case):
    """Level set for the oracle when no GPU set-up is at hand: the CPU
    oracle's own closest-point transform (reference algorithm)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    c = {k: v for k, v in case.items() if k not in ("init", "name")}
    c.update(threads=os.cpu_count() or 1)
    return orc.Oracle(c).get("lvset")


def run_cpu(case, lvset, steps, warmup, threads, sample_budget_s=None):
    """Time the CPU oracle on the workload; returns (cells*steps/s, steps, secs)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    o = orc.Oracle(oracle_case(case, lvset, threads))
    o.init(*wl.initial_state(case))
    if warmup:
        o.iterate(warmup)
    ncell = (len(case["xf"]) - 1) * (len(case["yf"]) - 1) * (len(case["zf"]) - 1)
    done, t0 = 0, time.perf_counter()
    while done < steps:
        o.iterate(1)
        done += 1
        if sample_budget_s is not None and time.perf_counter() - t0 > sample_budget_s:
            break
    secs = time.perf_counter() - t0
    return ncell * done / secs / 1e6, done, secs, o.stats()


def bench_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return 0
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    case = wl.sphere()
    threads = os.cpu_count() or 1
    lvset = cpu_level_set(case) if not args.lvset_from_gpu else None
    if lvset is None:
        ibm = importlib.import_module("2020researchproject_gb300")
        lvset = wl.build_solver(ibm, case).get_field("lvset")
    value, done, secs, st = run_cpu(case, lvset, args.steps, args.warmup, threads)
    line = {
        "metric": "Mcell-steps/s", "value": round(value, 4), "unit": "Mcell-steps/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": done, "warmup": args.warmup, "ms_per_step": round(secs / done * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": case["name"], "cells": 192 * 128 * 128, "triangles": 20480, "div_tol": DIV_TOL},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mcell-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{done} full fractional steps of the {case['name']} workload"},
        "e2e": {"value": round(value, 4), "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "oracle_stats": st,
    }
    print(json.dumps(line))
    return 0


def _profiler_range(on):
    """cudaProfilerStart/Stop around the headline timed region, so that
    `ncu --profile-from-start off` captures exactly its launches (no effect
    without a profiler)."""
    import ctypes
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        (rt.cudaProfilerStart if on else rt.cudaProfilerStop)()
        return


def _timed_arm(ibm, wl, case, precision, args, world, u0, headline=False):
    """Builds a solver for `case`, runs W warm-up steps and times K steps on
    the device (CUDA events on the solver's stream), sampling clocks.  The
    solver's iteration totals before and after the timed region give the
    mean Krylov iterations per timed step."""
    t0 = time.perf_counter()
    s = wl.build_solver(ibm, case, tol=MOM_TOL, div_tol=DIV_TOL)
    s.set_precision(ibm.MIXED32 if precision == "mixed" else ibm.FP64)
    if args.host_loop:
        s.set_graphs(False)
    setup_s = time.perf_counter() - t0
    s.init_flow_array(*u0)
    tuned = None
    if args.no_tune and precision == "mixed":
        s.set_precision(getattr(ibm, args.mixed_form))
    if args.no_tune and args.mg_sweeps:
        s.set_multigrid(*[int(v) for v in args.mg_sweeps.split(",")], 1.0)
    if not args.no_tune:
        # The autotuner picks the multigrid sweeps (and, for the mixed step,
        # which of the mixed solver forms) from the state after three
        # steps (past the start-up transient, whose harder solves favour
        # other settings), timing 8 steps per candidate (4-step trials
        # ranked sweeps that differ by 4 % in the timed steps either way
        # from one run to the next); the state is restored, and warm-up
        # follows.
        s.iterate(3)
        modes = ([("MIXED", ibm.MIXED), ("MIXED_MG", ibm.MIXED_MG), ("MIXED32", ibm.MIXED32)]
                 if precision == "mixed" else [("FP64", ibm.FP64)])
        trials = []
        for name, mode in modes:
            s.set_precision(mode)
            ms_t, sweeps = s.autotune(steps=8)
            trials.append((ms_t, name, mode, sweeps))
        ms_t, name, mode, sweeps = min(trials)
        s.set_precision(mode)
        s.set_multigrid(*sweeps, 1.0)
        tuned = {"mode": name, "mg_sweeps": list(sweeps),
                 "trials_ms_per_step": {t[1]: round(t[0], 2) for t in trials}}
    s.iterate(args.warmup)
    _barrier(world)
    l0 = ibm.kernel_launches()
    st0 = s.stats()
    gpu = 0 if world > 1 else int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0)
    with ClockSampler(gpu) as clk:
        if headline:
            _profiler_range(True)
        ms = s.time_iterate(args.steps)
        if headline:
            _profiler_range(False)
    launches = ibm.kernel_launches() - l0
    st = s.stats()
    n = max(1, st["steps_total"] - st0["steps_total"])
    iters = {"k_u": sum(st["iters_u_total"][l] - st0["iters_u_total"][l] for l in range(3)) / (3.0 * n),
             "k_p": (st["iters_p_total"] - st0["iters_p_total"]) / n,
             "max_div_over_timed_steps": st["max_div_max"]}
    ms = _barrier_max(ms, world)
    return {"solver": s, "ms": ms, "launches": launches, "launches_before": l0, "stats": st, "iters": iters,
            "clocks": clk.summary(), "setup_s": setup_s, "tuned": tuned}


def _vel_rel_l2(a, b):
    """Relative L2 difference of two velocity fields (u1, u2, u3 stacked),
    over cells finite in both."""
    num = den = 0.0
    for x, y in zip(a, b):
        m = np.isfinite(x) & np.isfinite(y)
        num += float(np.sum((x[m] - y[m]) ** 2))
        den += float(np.sum(y[m] ** 2))
    return (num / den) ** 0.5 if den > 0 else 0.0


def step_roofline(ms_per_step, cells, k_u, k_p, mixed, les, peak):
    """Step-level roofline from the algorithmic-bytes model of the step:
    B_step = 336 + 3 k_u 144 + k_p B_pois (+ 104 with LES) bytes per cell,
    B_pois = 492 with the FP64 multigrid, 318 with the FP32 one, with k_u
    and k_p the measured Krylov iterations per step (momentum per
    component, pressure)."""
    b_pois = 318.0 if mixed else 492.0
    b_step = 336.0 + 3 * k_u * 144.0 + k_p * b_pois + (104.0 if les else 0.0)
    ach = b_step * cells / (ms_per_step / 1e3) / 1e9
    return {"B_step": round(b_step, 1), "k_u": round(k_u, 2), "k_p": round(k_p, 2), "achieved": round(ach, 1),
            "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4)}


def e2e_loop(ibm, s, steps, world):
    """The metric end to end through the C ABI with pinned host buffers:
    per step, upload u1, u2, u3, p (IBMSolver_init_flow_array), one
    IBMSolver_iterate(1), read the four fields back (IBMSolver_get_field)."""
    fields = ["u1", "u2", "u3", "p"]
    host = [s.get_field(f) for f in fields]
    outs = [np.empty_like(h) for h in host]
    pinned = all(ibm.pin(a) for a in host + outs)
    _barrier(world)
    t1 = time.perf_counter()
    for _ in range(steps):
        s.init_flow_array(*host)
        s.iterate(1)
        for q, f in enumerate(fields):
            s.get_field_into(f, outs[q])
        host, outs = outs, host
    secs = _barrier_max(time.perf_counter() - t1, world)
    for a in host + outs:
        ibm.unpin(a)
    return secs, 4 * host[0].nbytes, pinned


def fp64_step_ops(arm):
    """FP64 operations (FMA = 2) of one step of `arm` (fp64 / mixed) on the
    sphere, from the committed ncu summary (profiles/fp64_step_ops.txt:
    '<arm> <workload> <ops> <momentum iterations> <pressure iterations>'
    of the profiled step), or None."""
    path = os.path.join(ROOT, "profiles", "fp64_step_ops.txt")
    try:
        for line in open(path):
            t = line.split()
            if len(t) >= 5 and not line.startswith("#") and t[0] == arm:
                return float(t[2]), float(t[3]), float(t[4])
    except OSError:
        pass
    return None


def fp64_roofline(arm, ms_per_step, fp64_tf):
    """The step against the FP64 pipe: the FP64 operations of a profiled
    step (ncu; its iteration counts are stated, close to the timed steps'
    means) over the measured time per step, as a fraction of the measured
    FP64 FMA rate."""
    rec = fp64_step_ops(arm)
    if rec is None:
        return None
    ops, it_u, it_p = rec
    tf = ops / (ms_per_step / 1e3) / 1e12
    return {"fp64_ops_per_step": ops, "achieved_tflops": round(tf, 3), "peak_tflops": round(fp64_tf, 3),
            "frac": round(tf / fp64_tf, 4), "peak_source": "measured FP64 FMA rate (fma_rate_tflops)",
            "ops_source": f"ncu, one profiled step ({it_u:g} momentum and {it_p:g} pressure iterations)"}


def fp64_ops_per_launch(kernel):
    """FP64 operations per launch (FMA = 2) of `kernel` from the committed
    ncu summary (profiles/fp64_ops.txt: '<kernel> <workload> <ops>'), or
    None."""
    path = os.path.join(ROOT, "profiles", "fp64_ops.txt")
    try:
        for line in open(path):
            t = line.split()
            if len(t) >= 3 and not line.startswith("#") and t[0] == kernel:
                return float(t[2])
    except OSError:
        pass
    return None


def error_vs_oracle(ibm, wl, case, u0, lvset, mixed_mode, steps=3):
    """Velocity and pressure error of the GPU steps against the CPU oracle
    (the restatement of the reference step, OpenMP on the host cores) from
    the same initial state after `steps` steps: the oracle and the FP64 step
    both solve to 1e-12; the mixed step and the FP64 step also at the
    benchmark's tolerances (momentum 1e-6, max|div U| <= 1e-8)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    t0 = time.perf_counter()
    o = orc.Oracle(oracle_case(case, lvset, os.cpu_count() or 1, div_tol=0.0, tol=1e-12))
    o.init(*u0)
    o.iterate(steps)
    ref_u = [o.get(f) for f in ("u1", "u2", "u3")]
    ref_p = o.get("p")
    oracle_s = time.perf_counter() - t0
    out = {"steps": steps, "oracle_tol": 1e-12, "oracle_seconds": round(oracle_s, 1)}

    def run(mode, tol, div_tol):
        sv = wl.build_solver(ibm, case, tol=tol, div_tol=div_tol)
        sv.set_precision(mode)
        sv.init_flow_array(*u0)
        sv.iterate(steps)
        e = {"velocity_rel_l2": _vel_rel_l2([sv.get_field(f) for f in ("u1", "u2", "u3")], ref_u),
             "pressure_rel_l2": _vel_rel_l2([sv.get_field("p")], [ref_p]),
             "max_div": sv.stats()["max_div_max"]}
        sv.close()
        return e

    out["fp64_tol_1e-12"] = run(ibm.FP64, 1e-12, 0.0)
    out["fp64_benchmark_tol"] = run(ibm.FP64, MOM_TOL, DIV_TOL)
    out["mixed_benchmark_tol"] = run(mixed_mode, MOM_TOL, DIV_TOL)
    return out


def bench_gb300(args):
    world, rank, local = _dist()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    ibm = importlib.import_module("2020researchproject_gb300")
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    case = {"sphere": wl.sphere, "cavity64": lambda: wl.cavity(64, 1000.0, 1e-3), "channel": wl.channel}[args.workload]()
    ncell = (len(case["xf"]) - 1) * (len(case["yf"]) - 1) * (len(case["zf"]) - 1)
    u0 = wl.initial_state(case)
    other = "fp64" if args.precision == "mixed" else "mixed"
    peak, peak_src = measured_peak_gbs()

    # --- device-timed region of the headline arm, then of the other arm
    # (same workload, same initial state, same step count).
    head = _timed_arm(ibm, wl, case, args.precision, args, world, u0, headline=True)
    print(f"[bench] {args.precision}: setup {head['setup_s']:.2f} s, {head['ms'] / args.steps:.2f} ms/step; timed "
          f"region started after {head['launches_before']} kernel launches", file=sys.stderr)
    s = head["solver"]
    value = world * ncell * args.steps / (head["ms"] / 1e3) / 1e6
    if args.profile_only:
        if rank == 0:
            print(json.dumps({"metric": "Mcell-steps/s", "value": round(value, 3), "unit": "Mcell-steps/s",
                              "profile_only": True, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": round(head["ms"] / args.steps, 3),
                              "gpu_launches": int(head["launches"]),
                              "launches_before_timed": int(head["launches_before"])}))
        return 0
    sec = _timed_arm(ibm, wl, case, other, args, world, u0)
    value2 = world * ncell * args.steps / (sec["ms"] / 1e3) / 1e6
    vel = [s.get_field(f) for f in ("u1", "u2", "u3")]
    vel2 = [sec["solver"].get_field(f) for f in ("u1", "u2", "u3")]
    mixed_arm, fp64_arm = (head, sec) if args.precision == "mixed" else (sec, head)
    err = _vel_rel_l2(vel, vel2)
    mixed_mode = getattr(ibm, (mixed_arm["tuned"] or {}).get("mode", args.mixed_form))

    # --- step-level roofline of both arms (measured iterations per step).
    roof_step = {a: step_roofline(arm["ms"] / args.steps, ncell, arm["iters"]["k_u"], arm["iters"]["k_p"],
                                  a == "mixed", False, peak)
                 for a, arm in (("mixed", mixed_arm), ("fp64", fp64_arm))}

    # --- stage profile (host-sequenced step, CUDA events per stage).
    s.set_profiling(True)
    s.iterate(2)
    prof = s.profile()
    s.set_profiling(False)

    # --- roofline of the dominant kernel: the fine-grid colour pass of the
    # pressure multigrid (FP32 in the mixed step, FP64 in the plain one),
    # back to back (as inside a V-cycle, L2-warm) and with the L2
    # overwritten before each launch (cold).
    k_ms, k_bytes = s.time_kernel("mg_color", reps=50)
    kc_ms, _ = s.time_kernel("mg_color", reps=20, cold=True)
    kname = "k_mg0_color_f32" if args.precision == "mixed" else "k_mg0_color_f64"
    ach_cold = k_bytes / (kc_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": f"{kname} (fine-grid Gauss-Seidel colour pass, pressure multigrid)",
            "achieved": round(ach_cold, 1), "peak": peak, "unit": "GB/s", "frac": round(ach_cold / peak, 4),
            "peak_source": peak_src, "traffic": traffic_per_launch(kname), "bytes_per_launch": k_bytes,
            "avg_launch_us": round(kc_ms * 1e3, 2), "timing": "cold L2 (256 MB written before each launch)",
            "warm": {"avg_launch_us": round(k_ms * 1e3, 2), "achieved": round(k_bytes / (k_ms / 1e3) / 1e9, 1),
                     "frac": round(k_bytes / (k_ms / 1e3) / 1e9 / peak, 4),
                     "timing": "back-to-back launches, L2-resident as inside a V-cycle"},
            "step": roof_step[args.precision]}
    sp_ms, sp_bytes = s.time_kernel("spmv_p", reps=50)
    spmv = {"achieved_gbs": round(sp_bytes / (sp_ms / 1e3) / 1e9, 1), "avg_launch_us": round(sp_ms * 1e3, 2),
            "bytes_per_launch": sp_bytes}

    # --- explicit stages of both arms: HBM fraction, and against the
    # measured FP64 FMA rate where the FP64 pipe bounds them.
    fp64_tf = ibm.measure_fma_rate(fp64=True)
    fp32_tf = ibm.measure_fma_rate(fp64=False)
    explicit = {}
    for a, arm in (("mixed", mixed_arm), ("fp64", fp64_arm)):
        sv = arm["solver"]
        ks = {}
        for kn in ("conv_rhs", "ustar_prhs", "update_next"):
            t_ms, t_b = sv.time_kernel(kn, reps=10, cold=True)
            e = {"avg_launch_us": round(t_ms * 1e3, 1), "bytes_per_launch": t_b,
                 "hbm_frac": round(t_b / (t_ms / 1e3) / 1e9 / peak, 4)}
            ops = fp64_ops_per_launch(("k_" + kn + ("32" if a == "mixed" else "")))
            if ops is not None:
                e["fp64_tflops"] = round(ops / (t_ms / 1e3) / 1e12, 3)
                e["fp64_frac"] = round(ops / (t_ms / 1e3) / 1e12 / fp64_tf, 4)
            ks[kn] = e
        explicit[a] = ks

    # --- end to end through the C ABI with pinned host buffers, both arms.
    e2e_s, bytes_io, pinned = e2e_loop(ibm, s, args.steps, world)
    e2e = world * ncell * args.steps / e2e_s / 1e6
    e2e2_s, _, _ = e2e_loop(ibm, sec["solver"], args.steps, world)
    e2e2 = world * ncell * args.steps / e2e2_s / 1e6

    st = head["stats"]
    line = {
        "metric": "Mcell-steps/s", "value": round(value, 3), "unit": "Mcell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(head["ms"] / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": case["name"], "cells": ncell, "triangles": 20480, "Re": case["re"],
                   "dt": case["dt"], "div_tol": DIV_TOL, "momentum_tol": MOM_TOL, "precision": args.precision,
                   "parallelism": f"replicas{world}", "l2": "working set > L2 (no flush needed)",
                   "steps_as": "host loop" if args.host_loop else "CUDA graph per step",
                   "setup_s": round(head["setup_s"], 2), "device": s.device_name(),
                   "autotuned": head["tuned"]},
        "e2e": {"value": round(e2e, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": bytes_io,
                "d2h_bytes_per_step": bytes_io, "pinned": pinned},
        "roofline": roof,
        "spmv_p": spmv,
        "gpu_launches": int(head["launches"]),
        "launches_before_timed": int(head["launches_before"]),
        "clocks": head["clocks"],
        other: {"value": round(value2, 3), "ms_per_step": round(sec["ms"] / args.steps, 3),
                "iters_p": sec["stats"]["iters_p"], "iters_u": sec["stats"]["iters_u"],
                "iters_per_step": sec["iters"], "max_div": sec["stats"]["max_div"], "autotuned": sec["tuned"],
                "gpu_launches": int(sec["launches"]), "clocks": sec["clocks"],
                "e2e": {"value": round(e2e2, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": bytes_io,
                        "d2h_bytes_per_step": bytes_io},
                "roofline_step": roof_step[other],
                "roofline_fp64": fp64_roofline(other, sec["ms"] / args.steps, fp64_tf)},
        "mixed_vs_fp64": round((mixed_arm["ms"] and fp64_arm["ms"] / mixed_arm["ms"]) or 0, 3),
        "error_vs_fp64": {"velocity_rel_l2": err, "max_div_mixed": mixed_arm["stats"]["max_div"],
                          "max_div_fp64": fp64_arm["stats"]["max_div"],
                          "note": f"after {args.warmup + args.steps} steps from the same state"},
        "solver": {"iters_p": st["iters_p"], "iters_u": st["iters_u"], "outer_p": st["outer_p"],
                   "iters_per_step": head["iters"], "max_div": st["max_div"], "mg_levels": st["mg_levels"]},
        "fma_rate_tflops": {"fp64": round(fp64_tf, 3), "fp32": round(fp32_tf, 2),
                            "how": "register-only FMA chains, 8 blocks of 256 per SM, best of 3"},
        "explicit_kernels": explicit,
        "roofline_fp64": fp64_roofline(args.precision, head["ms"] / args.steps, fp64_tf),
        "profile_ms": {k: [v[0], round(v[1], 3)] for k, v in sorted(prof.items())},
    }
    lv = s.get_field("lvset")
    s.close()
    head["solver"] = None
    sec["solver"].close()
    sec["solver"] = None
    def phase(name):   # marks the log, so that a solver warning can be placed
        print(f"[bench] {name}", file=sys.stderr, flush=True)

    if rank == 0 and world == 1 and not args.no_oracle:
        phase("error against the oracle")
        line["error_vs_oracle"] = error_vs_oracle(ibm, wl, case, u0, lv, mixed_mode)
    if rank == 0 and world == 1 and not args.no_extras:
        phase("configurations")
        line["configs"] = configs_arm(ibm, wl, args)
        phase("ensemble")
        line["ensemble"] = ensemble_arm(ibm, wl, args)
        phase("serving")
        line["serving"] = serving_arm(ibm, wl, args)
        phase("large-body set-up")
        line["large_body_setup"] = large_body_arm(ibm, wl)
    if rank == 0 and world == 1 and not args.no_cpu:
        # Past the first step (the start-up transient's pressure solves take
        # several times the iterations), as the reference arm's warm-up does.
        cv, done, secs, _ = run_cpu(case, lv, steps=3, warmup=1, threads=os.cpu_count() or 1, sample_budget_s=20)
        line["cpu_baseline"] = {"value": round(cv, 4), "unit": "Mcell-steps/s", "cores": os.cpu_count() or 1,
                                "kind": "port",
                                "sample": f"{done} fractional steps of the same {case['name']} workload after one "
                                          f"untimed step ({secs:.1f} s), CPU restatement of the reference step"}
    if rank == 0:
        print(json.dumps(line))
    return 0


def configs_arm(ibm, wl, args):
    """The other single-case configurations at their sizes, mixed (the
    FP32-stage step) and plain FP64: the 64^3 lid-driven cavity (200 steps
    from rest, Re 1000, dt 1e-3; its velocity error against the reference's
    own 200-step run solved to 1e-12, tests/golden/configs/c1_cavity64.npz)
    and the 128x96x128 channel LES (a 50-step sample of its 2000-step run,
    after 3 warm-up steps)."""
    out = {}
    ref = np.load(os.path.join(ROOT, "tests", "golden", "configs", "c1_cavity64.npz"))
    c1 = wl.cavity(64, 1000.0, 1e-3)
    cells = 64 ** 3
    r = {"workload": "cavity64 (Re 1000, dt 1e-3, lid u = 1)", "cells": cells, "steps": 200}
    for name, mode in (("mixed", ibm.MIXED32), ("fp64", ibm.FP64)):
        sv = wl.build_solver(ibm, c1, tol=MOM_TOL, div_tol=DIV_TOL)
        sv.set_precision(mode)
        sv.init_flow_array(*wl.initial_state(c1))
        sv.iterate(3)                                   # records the step graphs
        sv.init_flow_array(*wl.initial_state(c1))       # from rest again
        ms = sv.time_iterate(200)
        r[name] = round(cells * 200 / ms / 1e3, 3)
        r[name + "_error_vs_reference"] = _vel_rel_l2([sv.get_field(f) for f in ("u1", "u2", "u3")],
                                                      [ref[f] for f in ("u1", "u2", "u3")])
        r[name + "_max_div"] = sv.stats()["max_div_max"]
        sv.close()
    r["mixed_vs_fp64"] = round(r["mixed"] / r["fp64"], 3)
    out["cavity64"] = r
    c3 = wl.channel()
    cells = 128 * 96 * 128
    r = {"workload": "channel128x96x128 LES (Re_tau 180, Cs 0.1, dt 2e-3)", "cells": cells, "steps": 50,
         "sample": "50 of the 2000 steps, after 3 warm-up steps"}
    for name, mode in (("mixed", ibm.MIXED32), ("fp64", ibm.FP64)):
        sv = wl.build_solver(ibm, c3, tol=MOM_TOL, div_tol=DIV_TOL)
        sv.set_precision(mode)
        sv.init_flow_array(*wl.initial_state(c3))
        sv.iterate(3)
        ms = sv.time_iterate(50)
        r[name] = round(cells * 50 / ms / 1e3, 3)
        r[name + "_max_div"] = sv.stats()["max_div_max"]
        sv.close()
    r["mixed_vs_fp64"] = round(r["mixed"] / r["fp64"], 3)
    out["channel128x96x128"] = r
    return out


def ensemble_arm(ibm, wl, args, steps=300, alone_steps=30):
    """Batched ensemble (64 seeded immersed-body cases of uneven size, 300
    steps each): the mixed-precision batched step (one CUDA graph launch
    per step for all cases) and the FP64 batched step, against the plain
    FP64 step run case by case (rate from a 30-step sample of each case)."""
    cases = wl.ensemble()
    cells = sum((len(c["xf"]) - 1) * (len(c["yf"]) - 1) * (len(c["zf"]) - 1) for c in cases)
    out = {"cases": len(cases), "cells": cells, "steps": steps, "unit": "Mcell-steps/s",
           "workload": "64 cases, grids 32-96 x 32-64 x 32-64, boxes or spheres, Re 50-500, seed 2024"}
    for mode in ("mixed", "fp64"):
        solvers = []
        for c in cases:
            sv = wl.build_solver(ibm, c, tol=MOM_TOL, div_tol=DIV_TOL)
            sv.set_precision(ibm.MIXED32 if mode == "mixed" else ibm.FP64)
            sv.init_flow_array(*wl.initial_state(c))
            solvers.append(sv)
        b = ibm.Batch(solvers)
        b.iterate(1)
        ms = b.iterate(steps - 1)
        out[f"{mode}_batched"] = round(cells * (steps - 1) / ms / 1e3, 3)
        out[f"{mode}_batched_ms_per_step"] = round(ms / (steps - 1), 2)
        out[f"{mode}_max_div"] = max(sv.stats()["max_div_max"] for sv in solvers)
        if mode == "fp64":
            seq = 0.0
            for sv, c in zip(solvers, cases):
                sv.init_flow_array(*wl.initial_state(c))
                seq += sv.time_iterate(alone_steps)
            out["fp64_alone"] = round(cells * alone_steps / seq / 1e3, 3)
            out["fp64_alone_sample"] = f"{alone_steps} steps of each case from its initial state"
        del b
        for sv in solvers:
            sv.close()
    out["mixed_batched_vs_fp64_alone"] = round(out["mixed_batched"] / out["fp64_alone"], 3)
    out["mixed_batched_vs_fp64_batched"] = round(out["mixed_batched"] / out["fp64_batched"], 3)
    return out


def large_body_arm(ibm, wl):
    """Set-up at scale: assembly (closest-point transform, flags, ghost
    stencils, operators, multigrid) of the sphere192x128x128 grid around a
    dented body of 81,920 and 327,680 triangles, host wall time, after a
    first assembly of the same case (warm caches and context)."""
    out = {"grid": "192x128x128", "unit": "s"}
    for sub in (6, 7):
        case = wl.sphere()
        case["stl"] = wl.bumpy_stl(sub)
        times = []
        for _ in range(2):
            t0 = time.perf_counter()
            s = wl.build_solver(ibm, case, tol=MOM_TOL, div_tol=DIV_TOL)
            times.append(time.perf_counter() - t0)
            ghosts = len(s.ghost_stencils()[0])
            s.close()
        out[f"triangles_{20 * 4 ** sub}"] = {"assemble_s": round(times[-1], 3), "ghost_cells": ghosts}
    return out


def serving_arm(ibm, wl, args, njobs=20, alone_steps=10):
    """Continuous-batching server on the served stream's distribution:
    seeded Poisson arrivals at 20 jobs/s of cavity / sphere / box-cluster
    jobs, grids from 32^3 up to 256x128x128, Re 100-1000, 100-1000 steps (a
    seeded sample of `njobs` jobs of that stream), mixed precision (the
    FP32-stage step); p50/p99 job latency and aggregate throughput, against
    the same jobs run one by one on the plain FP64 step (device time of a
    10-step sample of each job, scaled to its step count)."""
    serve = importlib.import_module("2020researchproject_gb300.serve")
    jobs = serve.poisson_jobs(njobs=njobs, grid_max=(256, 128, 128), steps=(100, 1000))
    res = serve.Server(ibm, precision="mixed32").run(jobs)
    dev_ms = 0.0
    for j in jobs:
        sv = wl.build_solver(ibm, j.case, tol=MOM_TOL, div_tol=DIV_TOL)
        sv.set_precision(ibm.FP64)
        sv.init_flow_array(*wl.initial_state(j.case))
        sv.iterate(2)
        dev_ms += sv.time_iterate(alone_steps) * j.steps / alone_steps
        sv.close()
    alone = res["cell_steps"] / dev_ms / 1e3
    return {"jobs": njobs, "arrival_rate_per_s": 20.0,
            "workload": "cavity/sphere/box jobs, grids 32^3..256x128x128, 100-1000 steps, Re 100-1000, seed 4242 "
                        f"(the first {njobs} jobs of the stream)",
            "cell_steps": res["cell_steps"],
            "latency_p50_s": round(res["latency_p50_s"], 3), "latency_p99_s": round(res["latency_p99_s"], 3),
            "mcell_steps_per_s": round(res["mcell_steps_per_s"], 3), "max_active": res["max_active"],
            "wall_s": round(res["wall_s"], 2), "max_div": res["max_div"],
            "admission": res.get("admission"),
            "fp64_alone_device_mcell_steps_per_s": round(alone, 3),
            "served_vs_fp64_alone": round(res["mcell_steps_per_s"] / alone, 3)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other configurations, the ensemble and serving measurements")
    ap.add_argument("--no-oracle", action="store_true", help="skip the error against the CPU oracle")
    ap.add_argument("--no-tune", action="store_true", help="no autotuning: default (or the given) settings")
    ap.add_argument("--mixed-form", default="MIXED32", choices=["MIXED", "MIXED_MG", "MIXED32"],
                    help="with --no-tune: the mixed step's solver form")
    ap.add_argument("--mg-sweeps", default="", help="with --no-tune: multigrid sweeps 'pre,post,cpre,cpost,coarsest'")
    ap.add_argument("--host-loop", action="store_true",
                    help="host-sequenced steps instead of recorded graphs (same kernels; for ncu launch lists, "
                         "which do not list kernels inside graph loops)")
    ap.add_argument("--profile-only", action="store_true",
                    help="headline arm only (set-up, warm-up, timed region) for profiler runs")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                    help="arithmetic of the headline arm (the other one is measured beside it)")
    ap.add_argument("--workload", default="sphere", choices=["sphere", "cavity64", "channel"],
                    help="with --profile-only: the case of the profiled steps (the headline is the sphere)")
    ap.add_argument("--lvset-from-gpu", action="store_true",
                    help="reference arm: take the level set from the GPU set-up instead of the CPU transform")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.workload != "sphere" and not args.profile_only:
        ap.error("--workload selects the case of --profile-only runs")
    if args.impl == "reference":
        return bench_reference(args)
    return bench_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
