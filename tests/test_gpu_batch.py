"""Batched stepping (IBMBatch): many independent solvers advanced by one
CUDA graph launch per step.

A member of a batch must compute bit for bit what it computes alone
(same kernels, same order, on its own data), in both arithmetic modes,
whatever else is in the batch; members can join and leave between steps.
"""
import numpy as np
import pytest

from conftest import load_golden, package
from test_gpu_golden import build_case

pytestmark = pytest.mark.gpu

FIELDS = ["u1", "u2", "u3", "p", "U1", "pprime"]


def _fields(s):
    return {f: s.get_field(f) for f in FIELDS}


def _same(a, b):
    return all(np.array_equal(a[f], b[f], equal_nan=True) for f in FIELDS)


@pytest.mark.parametrize("combined", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed32"])
def test_batch_members_equal_solo_runs(precision, combined):
    ibm = package()
    names = ["cavity", "sphere", "channel_les", "mixed_box", "func_sphere"]
    cases = [load_golden(n) for n in names]
    mode = {"mixed": ibm.MIXED, "mixed32": ibm.MIXED32, "fp64": ibm.FP64}[precision]

    solo = []
    for c in cases:
        s = build_case(ibm, c, tol=1e-8)
        s.set_precision(mode)
        s.iterate(3)                      # one run of 3 steps
        solo.append((_fields(s), s.stats()))

    members = []
    for c in cases:
        s = build_case(ibm, c, tol=1e-8)
        s.set_precision(mode)
        members.append(s)
    batch = ibm.Batch(members, combined=combined)
    ms = batch.iterate(2)
    assert ms > 0
    batch.iterate(1)
    for name, s, (f0, st0) in zip(names, members, solo):
        st = s.stats()
        assert st["iter"] == 3
        assert _same(_fields(s), f0), f"{name}: batch member differs from the solo run"
        for k in ("iters_u", "iters_p", "res_p", "max_div"):
            assert st[k] == st0[k], f"{name} {k}: {st[k]} != {st0[k]}"


@pytest.mark.parametrize("combined", [True, False])
def test_batch_membership_changes_between_steps(combined):
    """A solver stepped partly alone, partly in a batch whose other members
    come and go, ends where the same runs alone end: its batched steps form
    one run from the moment it joined."""
    ibm = package()
    ref_case, other = load_golden("sphere"), load_golden("cavity")
    alone = build_case(ibm, ref_case, tol=1e-8)
    alone.iterate(1)
    alone.iterate(3)

    s = build_case(ibm, ref_case, tol=1e-8)
    t = build_case(ibm, other, tol=1e-8)
    s.iterate(1)                          # alone
    batch = ibm.Batch([s, t], combined=combined)
    batch.iterate(1)                      # with a partner
    batch.remove(t)
    batch.iterate(1)                      # partner gone
    u = build_case(ibm, other, tol=1e-8)
    batch.add(u)                          # a newcomer
    batch.iterate(1)
    assert s.stats()["iter"] == 4
    assert _same(_fields(s), _fields(alone))
    u_alone = build_case(ibm, other, tol=1e-8)
    u_alone.iterate(1)
    assert _same(_fields(u), _fields(u_alone))


def test_ensemble_cases_step_in_a_batch():
    """A few seeded ensemble cases (boxes and spheres, uneven grids) assemble
    and advance together, with the divergence logged for each."""
    ibm = package()
    wl = __import__("importlib").import_module("2020researchproject_gb300.workloads")
    cases = wl.ensemble(ncases=4, seed=11)
    solvers = []
    for c in cases:
        s = wl.build_solver(ibm, c, tol=1e-6, div_tol=1e-8)
        s.set_precision(ibm.MIXED)
        s.init_flow_array(*wl.initial_state(c))
        solvers.append(s)
    batch = ibm.Batch(solvers)
    batch.iterate(3)
    for c, s in zip(cases, solvers):
        st = s.stats()
        assert st["iter"] == 3
        assert st["max_div"] <= 1.001e-8, f"{c['name']}: max div {st['max_div']}"
        u = s.get_field("u1")
        assert np.isfinite(u[~np.isnan(u)]).all()
