"""Continuous-batching job server for the immersed-boundary time step.

Jobs (a case: grid, body, Reynolds number, boundary conditions; and a
step count) arrive over time.  The server admits queued jobs in arrival
order while their device footprint fits the HBM budget, keeps every
admitted job's fields and multigrid hierarchy resident on the GPU, and
advances all admitted jobs together, one batched step (one CUDA graph
launch, ``IBMBatch``) at a time.  A job that reaches its step count leaves
the batch and frees its memory; jobs that arrived meanwhile join at the
next step.  A job's result does not depend on what else ran with it: its
batched steps are one run, bitwise equal to stepping it alone.

Reported: per-job latency (arrival to completion), its p50/p99, and the
aggregate throughput in interior cell-steps per second.
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np

from . import geometry
from . import workloads as wl


@dataclasses.dataclass
class Job:
    id: int
    case: dict
    steps: int
    arrival: float                  # seconds after the start of the run
    cells: int = 0
    admitted: float | None = None
    finished: float | None = None
    done_steps: int = 0
    device_bytes: int = 0
    result: dict | None = None      # final fields, when kept
    result_stats: dict | None = None
    solver: object = None


def _cells(case):
    return (len(case["xf"]) - 1) * (len(case["yf"]) - 1) * (len(case["zf"]) - 1)


def _padded(case):
    return (len(case["xf"]) + 3) * (len(case["yf"]) + 3) * (len(case["zf"]) + 3)


def job_case(kind, nx, ny, nz, Re, rng):
    """A served case: a lid-driven cavity, flow past a sphere, or flow past
    a cluster of boxes, on an nx x ny x nz grid."""
    if kind == "cavity":
        return dict(name=f"cavity{nx}x{ny}x{nz}", xf=geometry.uniform_faces(0.0, 1.0, nx),
                    yf=geometry.uniform_faces(0.0, 1.0, ny), zf=geometry.uniform_faces(0.0, 1.0, nz), re=Re,
                    dt=0.25 / max(nx, ny, nz),
                    bc=["W wall", "E wall", "S wall", "N wall", "D wall", "U vel 1 0 0"], init=(0.0, 0.0, 0.0, 0.0))
    xf = geometry.uniform_faces(-4.0, 8.0, nx)
    yf = geometry.uniform_faces(-3.0, 3.0, ny)
    zf = geometry.uniform_faces(-3.0, 3.0, nz)
    h = min(12.0 / nx, 6.0 / ny, 6.0 / nz)
    if kind == "sphere":
        stl = wl.icosphere_stl(3, 0.5)
    else:
        boxes = wl._boxes(rng, int(rng.integers(1, 5)))
        stl = wl._body_stl("boxes", dict(boxes=boxes), ("boxes", tuple(boxes)))
    return dict(name=f"{kind}{nx}x{ny}x{nz}", xf=xf, yf=yf, zf=zf, re=Re, dt=0.25 * h,
                bc=["W vel 1 0 0", "E press 0", "S slip", "N slip", "D slip", "U slip"], stl=stl,
                init=(1.0, 0.0, 0.0, 0.0))


def poisson_jobs(njobs=40, rate=20.0, seed=4242, grid_max=(96, 64, 64), steps=(20, 100),
                 kinds=("cavity", "sphere", "boxes"), re=(100.0, 1000.0)):
    """Seeded Poisson arrivals (mean `rate` jobs/s) of cavity / sphere /
    box-cluster jobs with grids from 32^3 up to `grid_max`, Re ~ U[re] and
    step counts ~ U[steps]."""
    rng = np.random.Generator(np.random.Philox(seed))
    t = 0.0
    jobs = []
    for q in range(njobs):
        t += float(rng.exponential(1.0 / rate))
        kind = kinds[int(rng.integers(0, len(kinds)))]
        nx = int(rng.integers(32, grid_max[0] + 1))
        ny = int(rng.integers(32, grid_max[1] + 1))
        nz = int(rng.integers(32, grid_max[2] + 1))
        Re = float(rng.uniform(*re))
        case = job_case(kind, nx, ny, nz, Re, rng)
        n = int(rng.integers(steps[0], steps[1] + 1))
        jobs.append(Job(id=q, case=case, steps=n, arrival=t, cells=_cells(case)))
    return jobs


class Server:
    """Admits jobs by device footprint and advances the admitted ones in
    batched steps.  ``hbm_budget``: bytes the jobs may hold together (by
    default 80 % of the free device memory when the run starts);
    ``bytes_per_cell``: the footprint estimate per padded cell used before
    a job is assembled (raised to what admitted jobs actually take)."""

    def __init__(self, ibm, precision="mixed", tol=1e-6, div_tol=1e-8, hbm_budget=None, bytes_per_cell=1500.0,
                 keep_results=False, combined=False, overlap=True, admit_per_step=2):
        self.ibm = ibm
        # overlap: while the GPU runs a batched step (IBMBatch_launch ..
        # IBMBatch_wait) the host assembles at most `admit_per_step` queued
        # jobs, which join at the next step, so arrivals do not hold up the
        # resident jobs' steps; otherwise (or when nothing is resident) a job
        # is assembled before the step it joins.
        self.overlap = overlap
        self.admit_per_step = admit_per_step
        # False: each member steps through its own recorded graph (nothing is
        # re-recorded when jobs arrive or finish); True: one graph per
        # batched step, re-recorded on every membership change.
        self.combined = combined
        self.mode = {"mixed": ibm.MIXED, "mixed_mg": ibm.MIXED_MG, "mixed32": ibm.MIXED32,
                     "mixed32_ir": ibm.MIXED32_IR}.get(precision, ibm.FP64)
        self.tol, self.div_tol = tol, div_tol
        self.hbm_budget = hbm_budget
        self.bytes_per_cell = bytes_per_cell
        self.keep_results = keep_results

    def _estimate(self, job):
        return self.bytes_per_cell * _padded(job.case)

    def _admit(self, job, now):
        s = wl.build_solver(self.ibm, job.case, tol=self.tol, div_tol=self.div_tol)
        s.set_precision(self.mode)
        s.init_flow_array(*wl.initial_state(job.case))
        job.solver = s
        job.admitted = now
        job.device_bytes = s.device_bytes()
        if job.device_bytes > 0:
            self.bytes_per_cell = max(self.bytes_per_cell, job.device_bytes / _padded(job.case))
        return s

    def run(self, jobs, time_limit=600.0):
        """Serves `jobs` (arrival times relative to now); returns a summary."""
        budget = self.hbm_budget
        if budget is None:
            free = _free_device_bytes(self.ibm)
            budget = int(0.8 * free) if free else 64 << 30
        pending = collections.deque(sorted(jobs, key=lambda j: j.arrival))
        queue = collections.deque()
        active = []
        used = 0
        # Membership changes every few steps here, so each member steps
        # through its own recorded graph (nothing re-recorded on churn).
        batch = self.ibm.Batch(combined=self.combined)
        batched_steps = 0
        max_active = 0
        t0 = time.perf_counter()
        def admit_from_queue(limit):
            nonlocal used
            joined = []
            while queue and len(joined) < limit:
                if (active or joined) and used + self._estimate(queue[0]) > budget:
                    break
                job = queue.popleft()
                self._admit(job, time.perf_counter() - t0)
                used += job.device_bytes or self._estimate(job)
                joined.append(job)
            return joined

        def join(jobs_in):
            for job in jobs_in:
                batch.add(job.solver)
                active.append(job)

        while pending or queue or active:
            now = time.perf_counter() - t0
            if now > time_limit:
                raise RuntimeError("serving run exceeded its time limit")
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            if not active or not self.overlap:
                join(admit_from_queue(len(queue)))
            if not active:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 0.05)))
                continue
            max_active = max(max_active, len(active))
            joined = []
            if self.overlap:
                batch.launch()
                joined = admit_from_queue(self.admit_per_step)
                batch.wait()
            else:
                batch.iterate(1)
            batched_steps += 1
            for job in list(active):
                job.done_steps += 1
                if job.done_steps == job.steps:
                    job.finished = time.perf_counter() - t0
                    s = job.solver
                    if self.keep_results:
                        job.result = {f: s.get_field(f) for f in ("u1", "u2", "u3", "p")}
                    job.result_stats = s.stats()
                    batch.remove(s)
                    used -= job.device_bytes or self._estimate(job)
                    s.close()
                    job.solver = None
                    active.remove(job)
            join(joined)
        wall = time.perf_counter() - t0
        lat = np.array([j.finished - j.arrival for j in jobs])
        cell_steps = sum(j.cells * j.steps for j in jobs)
        return {"jobs": len(jobs), "wall_s": wall, "batched_steps": batched_steps, "max_active": max_active,
                "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                "latency_mean_s": float(lat.mean()), "cell_steps": cell_steps,
                "mcell_steps_per_s": cell_steps / wall / 1e6,
                "max_div": max(j.result_stats["max_div"] for j in jobs)}


def _free_device_bytes(ibm=None):
    if ibm is not None and hasattr(ibm, "load_library"):
        ibm.load_library()               # library first: its settings apply to the context
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so.13")
        free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
        if rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0:
            return free.value
    except OSError:
        pass
    return 0
