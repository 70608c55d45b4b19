"""Pressure multigrid coarsening (IBMSolver_set_coarsening).

* Halving every axis and coarsening by cell spacing both reproduce the
  reference's fixtures on stretched grids (the multigrid only
  preconditions: the converged fields are the same to 1e-9).
* On a uniform grid the two rules build the same levels: the steps are
  bitwise identical.
* On a stretched grid spacing coarsening keeps more cells per level (more
  levels) and needs fewer pressure iterations than halving.
"""
import importlib

import numpy as np
import pytest

from conftest import load_golden, rel_l2
from test_gpu_golden import FIELD_TOL, _MODES, _same_nan, build_case

pytestmark = pytest.mark.gpu


def _build(ibm, case, mode, ratio=0.0):
    """build_case with the coarsening set before assembly."""
    orig = ibm.IBMSolver.assemble

    def assemble(self):
        self.set_coarsening(mode, ratio)
        orig(self)

    ibm.IBMSolver.assemble = assemble
    try:
        return build_case(ibm, case, tol=case["meta"].get("solve_tol", 1e-12))
    finally:
        ibm.IBMSolver.assemble = orig


@pytest.mark.parametrize("precision", ["fp64", "mixed_mg"])
@pytest.mark.parametrize("name", ["sphere", "channel_les", "mixed_les", "bumpy_stl"])
def test_halving_matches_reference(ibm, name, precision):
    case = load_golden(name)
    s = _build(ibm, case, ibm.COARSEN_HALVE)
    s.set_precision(getattr(ibm, _MODES[precision]))
    for c, n in enumerate(case["meta"]["calls"], start=1):
        s.iterate(n)
        for f in ("u1", "u2", "u3", "p", "U1", "U2", "U3"):
            got, ref = s.get_field(f), case[f"{f}_{c}"]
            assert _same_nan(got, ref), f"{f} after call {c}: NaN mask differs"
            err = rel_l2(got, ref)
            assert err <= FIELD_TOL, f"{f} after call {c}: rel L2 {err:.3e}"


@pytest.mark.parametrize("ratio", [1.0, 2.5])
def test_spacing_ratio_matches_reference(ibm, ratio):
    case = load_golden("sphere")
    s = _build(ibm, case, ibm.COARSEN_SPACING, ratio)
    for c, n in enumerate(case["meta"]["calls"], start=1):
        s.iterate(n)
        for f in ("u1", "u2", "u3", "p"):
            assert rel_l2(s.get_field(f), case[f"{f}_{c}"]) <= FIELD_TOL, f


def test_uniform_grid_same_levels_bitwise():
    ibm = importlib.import_module("2020researchproject_gb300")
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    case = wl.sphere(nx=48, ny=32, nz=32)
    geo = importlib.import_module("2020researchproject_gb300.geometry")
    case["xf"] = geo.uniform_faces(-4.0, 8.0, 48)
    case["yf"] = geo.uniform_faces(-4.0, 4.0, 32)
    case["zf"] = geo.uniform_faces(-4.0, 4.0, 32)
    u0 = wl.initial_state(case)
    out = []
    for mode in (ibm.COARSEN_HALVE, ibm.COARSEN_SPACING):
        s = wl.build_solver(ibm, case, tol=1e-6, div_tol=1e-8, coarsening=mode)
        s.set_precision(ibm.MIXED_MG)
        s.init_flow_array(*u0)
        s.iterate(3)
        out.append(({f: s.get_field(f) for f in ("u1", "u2", "u3", "p")}, s.stats()))
        s.close()
    (a, sa), (b, sb) = out
    assert sa["mg_levels"] == sb["mg_levels"] and sa["iters_p"] == sb["iters_p"]
    for f in a:
        assert np.array_equal(a[f], b[f], equal_nan=True), f


def test_spacing_needs_fewer_iterations_on_stretched_grid():
    ibm = importlib.import_module("2020researchproject_gb300")
    wl = importlib.import_module("2020researchproject_gb300.workloads")
    case = wl.sphere(nx=96, ny=64, nz=64, subdivisions=3)
    u0 = wl.initial_state(case)
    st = {}
    for mode in (ibm.COARSEN_HALVE, ibm.COARSEN_SPACING):
        s = wl.build_solver(ibm, case, tol=1e-6, div_tol=1e-8, coarsening=mode)
        s.set_precision(ibm.FP64)
        s.init_flow_array(*u0)
        s.iterate(3)
        st[mode] = s.stats()
        assert st[mode]["max_div"] <= 1.001e-8
        s.close()
    assert st[ibm.COARSEN_SPACING]["mg_levels"] >= st[ibm.COARSEN_HALVE]["mg_levels"]
    assert st[ibm.COARSEN_SPACING]["iters_p"] < st[ibm.COARSEN_HALVE]["iters_p"]


def test_coarsening_arguments_checked(ibm):
    case = load_golden("sphere")
    s = build_case(ibm, case)
    with pytest.raises(ibm.IBM3DError, match="before IBMSolver_assemble"):
        s.set_coarsening(ibm.COARSEN_HALVE)
    t = ibm.IBMSolver()
    with pytest.raises(ibm.IBM3DError, match="unknown mode"):
        t.set_coarsening(7)
    with pytest.raises(ibm.IBM3DError, match="width ratio"):
        t.set_coarsening(ibm.COARSEN_SPACING, 0.5)
