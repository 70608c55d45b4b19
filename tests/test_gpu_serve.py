"""Serving on the GPU: jobs that arrive while others run join the batched
step as memory frees up, and each job's result is the same in the mix as
alone (bitwise: its batched steps are one run of its own kernels on its own
data)."""
import importlib

import numpy as np
import pytest

from conftest import package

pytestmark = pytest.mark.gpu


def test_served_jobs_equal_jobs_run_alone():
    ibm = package()
    serve = importlib.import_module("2020researchproject_gb300.serve")
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    # Enough steps per job that later jobs arrive while earlier ones step.
    jobs = serve.poisson_jobs(njobs=6, rate=40.0, seed=77, grid_max=(48, 40, 40), steps=(20, 30))
    for j in jobs:                        # arrivals 10 ms apart: later jobs find earlier ones running
        j.arrival = 0.01 * j.id
    # A budget that holds any two jobs but not every three, so that later
    # jobs wait and join the batch as earlier ones leave.
    sizes, per_cell = [], 0.0
    for j in jobs:
        probe = wl.build_solver(ibm, j.case)
        sizes.append(probe.device_bytes())
        padded = (len(j.case["xf"]) + 3) * (len(j.case["yf"]) + 3) * (len(j.case["zf"]) + 3)
        per_cell = max(per_cell, sizes[-1] / padded)
        probe.close()
    top = sorted(sizes)[-2:]
    srv = serve.Server(ibm, precision="mixed", hbm_budget=int(sum(top) * 1.02), bytes_per_cell=per_cell,
                       keep_results=True)
    out = srv.run(jobs, time_limit=300)
    assert out["jobs"] == 6 and out["max_active"] >= 2
    for j in jobs:
        assert 0 < j.result_stats["max_div"] <= 1.001e-8, f"job {j.id}: max div {j.result_stats['max_div']}"
        s = wl.build_solver(ibm, j.case, tol=1e-6, div_tol=1e-8)
        s.set_precision(ibm.MIXED)
        s.init_flow_array(*wl.initial_state(j.case))
        s.iterate(j.steps)
        for f in ("u1", "u2", "u3", "p"):
            assert np.array_equal(s.get_field(f), j.result[f], equal_nan=True), \
                f"job {j.id} ({j.case['name']}): {f} differs between the served run and the run alone"
        s.close()
