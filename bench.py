#!/usr/bin/env python
"""Benchmark of the immersed-boundary fractional step on GB300.

Workload: flow past a sphere, 192x128x128 cells (3,145,728 interior cells),
body-clustered grid on [-5,15]x[-5,5]^2, 20480-triangle icosphere r = 0.5,
Re 300, dt 5e-3, uniform inflow, pressure outlet, free-slip sides; the
pressure solve runs to max|div U^{n+1}| <= 1e-8 on fluid cells every step,
momentum to the reference drivers' relative tolerance 1e-6.  Synthetic,
seeded inputs (the reference has no public dataset).

Metric: Mcell-steps/s = interior cells x steps / seconds, for the
mixed-precision step (FP32 Krylov/multigrid inner solves inside FP64
iterative refinement, everything else FP64), with the plain FP64 step
measured beside it on the same state ("fp64", "mixed_vs_fp64") and the
velocity difference between the two after the run ("error_vs_fp64").
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
    the device (CUDA events on the solver's stream), sampling clocks."""
    t0 = time.perf_counter()
    s = wl.build_solver(ibm, case, tol=MOM_TOL, div_tol=DIV_TOL)
    s.set_precision(ibm.MIXED if precision == "mixed" else ibm.FP64)
    if args.host_loop:
        s.set_graphs(False)
    setup_s = time.perf_counter() - t0
    s.init_flow_array(*u0)
    tuned = None
    if args.no_tune and precision == "mixed" and args.mixed_form == "MIXED_MG":
        s.set_precision(ibm.MIXED_MG)
    if args.no_tune and args.mg_sweeps:
        s.set_multigrid(*[int(v) for v in args.mg_sweeps.split(",")], 1.0)
    if not args.no_tune:
        # The autotuner picks the multigrid sweeps (and, for the mixed step,
        # which of the two mixed solver forms) from the state after three
        # steps (past the start-up transient, whose harder solves favour
        # other settings); the state is restored, and warm-up follows.
        s.iterate(3)
        modes = [("MIXED", ibm.MIXED), ("MIXED_MG", ibm.MIXED_MG)] if precision == "mixed" else [("FP64", ibm.FP64)]
        trials = []
        for name, mode in modes:
            s.set_precision(mode)
            ms_t, sweeps = s.autotune(steps=4)
            trials.append((ms_t, name, mode, sweeps))
        ms_t, name, mode, sweeps = min(trials)
        s.set_precision(mode)
        s.set_multigrid(*sweeps, 1.0)
        tuned = {"mode": name, "mg_sweeps": list(sweeps),
                 "trials_ms_per_step": {t[1]: round(t[0], 2) for t in trials}}
    s.iterate(args.warmup)
    _barrier(world)
    l0 = ibm.kernel_launches()
    gpu = 0 if world > 1 else int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0)
    with ClockSampler(gpu) as clk:
        if headline:
            _profiler_range(True)
        ms = s.time_iterate(args.steps)
        if headline:
            _profiler_range(False)
    launches = ibm.kernel_launches() - l0
    ms = _barrier_max(ms, world)
    return {"solver": s, "ms": ms, "launches": launches, "launches_before": l0, "stats": s.stats(),
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


def bench_gb300(args):
    world, rank, local = _dist()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    ibm = importlib.import_module("2020researchproject_gb300")
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    case = wl.sphere()
    ncell = (len(case["xf"]) - 1) * (len(case["yf"]) - 1) * (len(case["zf"]) - 1)
    u0 = wl.initial_state(case)
    other = "fp64" if args.precision == "mixed" else "mixed"

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
    del sec["solver"]

    # --- stage profile (host-sequenced step, CUDA events per stage).
    s.set_profiling(True)
    s.iterate(2)
    prof = s.profile()
    s.set_profiling(False)

    # --- roofline of the dominant kernel: the fine-grid colour pass of the
    # pressure multigrid (FP32 in the mixed step, FP64 in the plain one).
    peak, peak_src = measured_peak_gbs()
    k_ms, k_bytes = s.time_kernel("mg_color", reps=50)
    ach = k_bytes / (k_ms / 1e3) / 1e9
    kname = "k_mg0_color_f32" if args.precision == "mixed" else "k_mg0_color_f64"
    roof = {"bound": "hbm", "kernel": f"{kname} (fine-grid Gauss-Seidel colour pass, pressure multigrid)",
            "achieved": round(ach, 1), "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4),
            "peak_source": peak_src, "traffic": traffic_per_launch(kname),
            "bytes_per_launch": k_bytes, "avg_launch_us": round(k_ms * 1e3, 2)}
    sp_ms, sp_bytes = s.time_kernel("spmv_p", reps=50)
    spmv = {"achieved_gbs": round(sp_bytes / (sp_ms / 1e3) / 1e9, 1), "avg_launch_us": round(sp_ms * 1e3, 2),
            "bytes_per_launch": sp_bytes}

    # --- end to end through the C ABI with pinned host buffers.
    fields = ["u1", "u2", "u3", "p"]
    host = [s.get_field(f) for f in fields]
    outs = [np.empty_like(h) for h in host]
    pinned = all(ibm.pin(a) for a in host + outs)
    _barrier(world)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        s.init_flow_array(*host)
        s.iterate(1)
        for q, f in enumerate(fields):
            s.get_field_into(f, outs[q])
        host, outs = outs, host
    e2e_s = _barrier_max(time.perf_counter() - t1, world)
    e2e = world * ncell * args.steps / e2e_s / 1e6
    bytes_io = 4 * host[0].nbytes

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
                "iters_p": sec["stats"]["iters_p"], "max_div": sec["stats"]["max_div"], "autotuned": sec["tuned"],
                "gpu_launches": int(sec["launches"]), "clocks": sec["clocks"]},
        "mixed_vs_fp64": round((mixed_arm["ms"] and fp64_arm["ms"] / mixed_arm["ms"]) or 0, 3),
        "error_vs_fp64": {"velocity_rel_l2": err, "max_div_mixed": mixed_arm["stats"]["max_div"],
                          "max_div_fp64": fp64_arm["stats"]["max_div"],
                          "note": f"after {args.warmup + args.steps} steps from the same state"},
        "solver": {"iters_p": st["iters_p"], "iters_u": st["iters_u"], "outer_p": st["outer_p"],
                   "max_div": st["max_div"], "mg_levels": st["mg_levels"]},
        "profile_ms": {k: [v[0], round(v[1], 3)] for k, v in sorted(prof.items())},
    }
    lv = s.get_field("lvset")
    s.close()
    head["solver"] = None
    if rank == 0 and world == 1 and not args.no_extras:
        line["ensemble"] = ensemble_arm(ibm, wl, args)
        line["serving"] = serving_arm(ibm, wl, args)
        line["large_body_setup"] = large_body_arm(ibm, wl)
    if rank == 0 and world == 1 and not args.no_cpu:
        cv, done, secs, _ = run_cpu(case, lv, steps=2, warmup=0, threads=os.cpu_count() or 1, sample_budget_s=25)
        line["cpu_baseline"] = {"value": round(cv, 4), "unit": "Mcell-steps/s", "cores": os.cpu_count() or 1,
                                "kind": "port",
                                "sample": f"{done} fractional steps of the same {case['name']} workload "
                                          f"({secs:.1f} s), CPU restatement of the reference step"}
    if rank == 0:
        print(json.dumps(line))
    return 0


def ensemble_arm(ibm, wl, args, steps=5):
    """Batched ensemble (64 seeded immersed-body cases of uneven size): the
    mixed-precision batched step (one CUDA graph launch per step for all
    cases) against the plain FP64 step run case by case, and the FP64
    batched step."""
    cases = wl.ensemble()
    cells = sum((len(c["xf"]) - 1) * (len(c["yf"]) - 1) * (len(c["zf"]) - 1) for c in cases)
    out = {"cases": len(cases), "cells": cells, "steps": steps, "unit": "Mcell-steps/s",
           "workload": "64 cases, grids 32-96 x 32-64 x 32-64, boxes or spheres, Re 50-500, seed 2024"}
    for mode in ("mixed", "fp64"):
        solvers = []
        for c in cases:
            sv = wl.build_solver(ibm, c, tol=MOM_TOL, div_tol=DIV_TOL)
            # mixed: the FP64-Krylov / FP32-multigrid form (faster than the
            # refinement form on these cases: 82 against 76 Mcell-steps/s)
            sv.set_precision(ibm.MIXED_MG if mode == "mixed" else ibm.FP64)
            sv.init_flow_array(*wl.initial_state(c))
            solvers.append(sv)
        b = ibm.Batch(solvers)
        b.iterate(1)
        ms = b.iterate(steps)
        out[f"{mode}_batched"] = round(cells * steps / ms / 1e3, 3)
        out[f"{mode}_batched_ms_per_step"] = round(ms / steps, 2)
        out[f"{mode}_max_div"] = max(sv.stats()["max_div"] for sv in solvers)
        if mode == "fp64":
            seq = sum(sv.time_iterate(steps) for sv in solvers)
            out["fp64_alone"] = round(cells * steps / seq / 1e3, 3)
        del b
        for sv in solvers:
            sv.close()
    out["mixed_batched_vs_fp64_alone"] = round(out["mixed_batched"] / out["fp64_alone"], 3)
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


def serving_arm(ibm, wl, args, njobs=32, steps=(100, 300)):
    """Continuous-batching server on seeded Poisson arrivals (20 jobs/s):
    cavity / sphere / box-cluster jobs, grids 32^3 to 96x64x64, 100-300
    steps (the low end of the 100-1000 of the served stream, so that the
    run ends in seconds while the GPU, not the arrival process, bounds the
    throughput), mixed precision (FP64 Krylov, FP32 multigrid); p50/p99 job
    latency and aggregate throughput, against the same jobs run one by one
    on the plain FP64 step."""
    serve = importlib.import_module("2020researchproject_gb300.serve")
    jobs = serve.poisson_jobs(njobs=njobs, steps=steps)
    res = serve.Server(ibm, precision="mixed_mg").run(jobs)
    dev_ms = 0.0
    for j in jobs:
        sv = wl.build_solver(ibm, j.case, tol=MOM_TOL, div_tol=DIV_TOL)
        sv.set_precision(ibm.FP64)
        sv.init_flow_array(*wl.initial_state(j.case))
        dev_ms += sv.time_iterate(j.steps)
        sv.close()
    alone = res["cell_steps"] / dev_ms / 1e3
    return {"jobs": njobs, "arrival_rate_per_s": 20.0,
            "workload": f"cavity/sphere/box jobs, grids 32^3..96x64x64, {steps[0]}-{steps[1]} steps, Re 100-1000, "
                        "seed 4242",
            "latency_p50_s": round(res["latency_p50_s"], 3), "latency_p99_s": round(res["latency_p99_s"], 3),
            "mcell_steps_per_s": round(res["mcell_steps_per_s"], 3), "max_active": res["max_active"],
            "wall_s": round(res["wall_s"], 2), "max_div": res["max_div"],
            "fp64_alone_device_mcell_steps_per_s": round(alone, 3),
            "served_vs_fp64_alone": round(res["mcell_steps_per_s"] / alone, 3)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true", help="skip the ensemble and serving measurements")
    ap.add_argument("--no-tune", action="store_true", help="no autotuning: default (or the given) settings")
    ap.add_argument("--mixed-form", default="MIXED", choices=["MIXED", "MIXED_MG"],
                    help="with --no-tune: the mixed step's solver form")
    ap.add_argument("--mg-sweeps", default="", help="with --no-tune: multigrid sweeps 'pre,post,cpre,cpost,coarsest'")
    ap.add_argument("--host-loop", action="store_true",
                    help="host-sequenced steps instead of recorded graphs (same kernels; for ncu launch lists, "
                         "which do not list kernels inside graph loops)")
    ap.add_argument("--profile-only", action="store_true",
                    help="headline arm only (set-up, warm-up, timed region) for profiler runs")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                    help="arithmetic of the headline arm (the other one is measured beside it)")
    ap.add_argument("--lvset-from-gpu", action="store_true",
                    help="reference arm: take the level set from the GPU set-up instead of the CPU transform")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return bench_reference(args)
    return bench_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
