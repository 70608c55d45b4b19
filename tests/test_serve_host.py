"""Host logic of the continuous-batching server (no GPU): admission in
arrival order by device footprint, batched stepping, departures, and the latency summary,
driven through a fake of the library's solver/batch API."""
import importlib
import time

import numpy as np

serve = importlib.import_module("2020researchproject_gb300.serve")


class FakeSolver:
    made = []

    def __init__(self):
        self.iter = 0
        self.closed = False
        self.padded = 0
        FakeSolver.made.append(self)

    def __getattr__(self, name):          # set_bc, set_params, assemble, ... accept anything
        if name.startswith("set_") or name == "assemble":
            return lambda *a, **k: None
        raise AttributeError(name)

    def set_grid(self, xf, yf, zf):
        self.padded = (len(xf) + 3) * (len(yf) + 3) * (len(zf) + 3)

    def init_flow_array(self, *a):
        pass

    def device_bytes(self):
        return 100 * self.padded

    def stats(self):
        return {"iter": self.iter, "max_div": 1e-9}

    def get_field(self, name):
        return np.full(3, float(self.iter))

    def close(self):
        self.closed = True


class FakeBatch:
    log = []

    def __init__(self, members=(), combined=True):
        self.members = list(members)

    def add(self, s):
        self.members.append(s)
        FakeBatch.log.append(("add", id(s)))

    def remove(self, s):
        self.members.remove(s)
        FakeBatch.log.append(("remove", id(s)))

    def iterate(self, n=1):
        time.sleep(0.02)                   # a step takes a while
        FakeBatch.log.append(("step", len(self.members)))
        for m in self.members:
            m.iter += n
        return 1.0

    def launch(self):                      # a step in two halves: members are fixed in between
        self.launched = list(self.members)
        FakeBatch.log.append(("launch", len(self.members)))

    def wait(self):
        time.sleep(0.02)
        assert self.launched == self.members, "membership changed while a step was in flight"
        FakeBatch.log.append(("step", len(self.members)))
        for m in self.members:
            m.iter += 1


class FakeIBM:
    MIXED, FP64 = 1, 0
    SOLVER_BiCGSTAB, PRECOND_AMG = 2, 1
    IBMSolver = FakeSolver
    Batch = FakeBatch

    class Polyhedron:
        def __init__(self, path):
            self.path = path

    def __getattr__(self, name):          # DIR_* / BC_* constants
        return 0


def _jobs():
    rng = np.random.Generator(np.random.Philox(1))
    jobs = []
    for q, (n, steps) in enumerate([(32, 3), (40, 2), (36, 4)]):
        case = serve.job_case("cavity", n, n, n, 100.0, rng)
        jobs.append(serve.Job(id=q, case=case, steps=steps, arrival=0.0, cells=n ** 3))
    return jobs


def test_server_admits_by_footprint_and_finishes_every_job():
    FakeSolver.made.clear()
    FakeBatch.log.clear()
    jobs = _jobs()
    # Budget for the first two jobs only: the third waits for a departure.
    pad = [(len(j.case["xf"]) + 3) ** 3 for j in jobs]
    budget = 100 * (pad[0] + pad[1]) + 1
    srv = serve.Server(FakeIBM(), hbm_budget=budget, bytes_per_cell=100.0, keep_results=True)
    out = srv.run(jobs)
    assert out["jobs"] == 3 and out["max_active"] == 2
    for j in jobs:
        assert j.done_steps == j.steps and j.finished >= j.arrival
        assert j.result["u1"][0] == j.steps        # stepped exactly its own count
    assert all(s.closed for s in FakeSolver.made)
    adds = [i for i, e in enumerate(FakeBatch.log) if e[0] == "add"]
    assert len(adds) == 3
    # the third job joined only after the second (2 steps) left
    first_remove = next(i for i, e in enumerate(FakeBatch.log) if e[0] == "remove")
    assert adds[2] > first_remove
    assert out["latency_p50_s"] <= out["latency_p99_s"]
    assert out["cell_steps"] == sum(j.cells * j.steps for j in jobs)


def test_poisson_jobs_are_seeded_and_bounded():
    a = serve.poisson_jobs(njobs=12, rate=20.0, seed=5, grid_max=(48, 40, 40), steps=(5, 9))
    b = serve.poisson_jobs(njobs=12, rate=20.0, seed=5, grid_max=(48, 40, 40), steps=(5, 9))
    assert [j.arrival for j in a] == [j.arrival for j in b]
    assert all(np.diff([j.arrival for j in a]) > 0)
    for j in a:
        nx, ny, nz = (len(j.case[k]) - 1 for k in ("xf", "yf", "zf"))
        assert 32 <= nx <= 48 and 32 <= ny <= 40 and 32 <= nz <= 40 and 5 <= j.steps <= 9


def test_setup_failure_reaches_the_caller():
    class Broken(FakeIBM):
        class IBMSolver(FakeSolver):
            def assemble(self):
                raise RuntimeError("assembly failed")

    srv = serve.Server(Broken(), hbm_budget=1 << 40, bytes_per_cell=100.0)
    try:
        srv.run(_jobs(), time_limit=30)
    except RuntimeError as e:
        assert "assembly failed" in str(e)
    else:
        raise AssertionError("the set-up error was swallowed")


def test_arrivals_are_assembled_while_the_gpu_steps():
    """A job that arrives while others are resident is assembled between
    the launch of a batched step and its wait (the GPU keeps stepping the
    resident jobs) and joins at the next step."""
    class Logged(FakeIBM):
        class IBMSolver(FakeSolver):
            def assemble(self):
                FakeBatch.log.append(("assemble", id(self)))

    FakeSolver.made.clear()
    FakeBatch.log.clear()
    rng = np.random.Generator(np.random.Philox(2))
    jobs = [serve.Job(id=0, case=serve.job_case("cavity", 32, 32, 32, 100.0, rng), steps=6, arrival=0.0,
                      cells=32 ** 3),
            serve.Job(id=1, case=serve.job_case("cavity", 36, 36, 36, 100.0, rng), steps=2, arrival=0.03,
                      cells=36 ** 3)]
    out = serve.Server(Logged(), hbm_budget=1 << 40, bytes_per_cell=100.0).run(jobs)
    assert out["jobs"] == 2
    log = FakeBatch.log
    a1 = [i for i, e in enumerate(log) if e[0] == "assemble"][1]
    assert log[a1 - 1][0] == "launch" and log[a1 + 1][0] == "step"   # inside a step in flight
    assert all(j.done_steps == j.steps for j in jobs)
