"""Recorded (CUDA-graph) time steps against host-sequenced ones.

With graphs on, a step runs as one graph whose Krylov loops iterate on the
device (conditional while nodes); with graphs off the host launches every
kernel and reads the solver scalars after each half iteration.  The two
must agree bit for bit, in both arithmetic modes, including the iteration
counts and the logged divergence.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from test_gpu_golden import build_case

pytestmark = pytest.mark.gpu

FIELDS = ["u1", "u2", "u3", "p", "U1", "U2", "U3", "pprime", "u1star"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", [n for n in golden_cases() if n in ("sphere", "channel_les", "cavity", "func_sphere")])
def test_graph_equals_host_loop(ibm, name, precision):
    case = load_golden(name)
    out = []
    for graphs in (True, False):
        s = build_case(ibm, case, tol=1e-8)
        s.set_precision(ibm.MIXED if precision == "mixed" else ibm.FP64)
        s.set_graphs(graphs)
        stats = []
        for _ in range(3):
            s.iterate(1)
            stats.append(s.stats())
        out.append(({f: s.get_field(f) for f in FIELDS}, stats))
    (fa, sa), (fb, sb) = out
    for f in FIELDS:
        assert np.array_equal(fa[f], fb[f], equal_nan=True), f"{f} differs between graph and host loop"
    for a, b in zip(sa, sb):
        for k in ("iters_u", "iters_p", "res_u", "res_p", "max_div", "outer_u", "outer_p"):
            assert a[k] == b[k], f"{k}: {a[k]} != {b[k]}"


@pytest.mark.parametrize("precision", ["fp64", "mixed_mg"])
@pytest.mark.parametrize("solver", ["bicgstab", "gmres"])
def test_graph_equals_host_loop_other_solvers(ibm, solver, precision):
    """The FP64-Krylov / FP32-multigrid mode and SOLVER_GMRES record and
    replay bit for bit too (fresh solvers: the result depends on the second
    field buffers, so both runs start from the same state)."""
    case = load_golden("sphere")
    out = []
    for graphs in (True, False):
        s = build_case(ibm, case, tol=1e-8)
        if solver == "gmres":
            s.set_linear_solver(ibm.SOLVER_GMRES, ibm.PRECOND_AMG, 1e-8)
            s.set_gmres_restart(8)
        s.set_precision(ibm.MIXED_MG if precision == "mixed_mg" else ibm.FP64)
        s.set_graphs(graphs)
        stats = []
        for _ in range(3):
            s.iterate(1)
            stats.append(s.stats())
        out.append(({f: s.get_field(f) for f in FIELDS}, stats))
    (fa, sa), (fb, sb) = out
    for f in FIELDS:
        assert np.array_equal(fa[f], fb[f], equal_nan=True), f"{f} differs between graph and host loop"
    for a, b in zip(sa, sb):
        for k in ("iters_u", "iters_p", "res_p", "max_div", "outer_p"):
            assert a[k] == b[k], f"{k}: {a[k]} != {b[k]}"


@pytest.mark.parametrize("precision", ["MIXED", "MIXED32"])
def test_autotune_leaves_the_run_unchanged(ibm, precision):
    """The autotuner times candidate sweep settings from the current state
    and restores it: a run continued after tuning equals the same run with
    the chosen setting and no tuning."""
    case = load_golden("sphere")
    a = build_case(ibm, case, tol=1e-8)
    a.set_precision(getattr(ibm, precision))
    a.iterate(1)
    ms, best = a.autotune(steps=1)
    assert ms > 0 and len(best) == 5
    assert a.stats()["iter"] == 1
    a.iterate(2)
    b = build_case(ibm, case, tol=1e-8)
    b.set_precision(getattr(ibm, precision))
    b.iterate(1)
    b.set_multigrid(*best, 1.0)
    b.iterate(2)
    for f in FIELDS:
        assert np.array_equal(a.get_field(f), b.get_field(f), equal_nan=True), f
