"""GPU parity against the golden fixtures made by running the reference.

Each fixture (tests/golden/*.npz, written by tests/golden/make_golden.py
from the reference's own C sources) holds a small case's inputs and the
reference's outputs after assembly and after each IBMSolver_iterate call.
The GPU path runs the same case through the C ABI and must reproduce

* flags, level set, p_coeffsum and ghost stencils (indices and raw
  weights) bit for bit;
* u, p, face velocities and the last step's u*, U*, p', N within 1e-9
  relative L2, with identical NaN masks (both sides solve to tol 1e-12),
  in both arithmetic modes: the plain FP64 solves and the mixed path
  (FP64 iterative refinement around FP32 BiCGSTAB + FP32 multigrid), which
  stops on the same FP64 residual criterion.
"""
import os

import numpy as np
import pytest

import valfuncs
from conftest import GOLDEN, case_stl, golden_cases, load_golden, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-9
PPRIME_TOL = 1e-8

_BC = {"vel": "BC_VELOCITY_COMPONENT", "press": "BC_PRESSURE", "wall": "BC_STATIONARY_WALL",
       "slip": "BC_FREE_SLIP_WALL", "sym": "BC_SYMMETRIC", "per": "BC_ALL_PERIODIC",
       "velper": "BC_VELOCITY_PERIODIC"}
_DIR = {"N": "DIR_NORTH", "E": "DIR_EAST", "S": "DIR_SOUTH", "W": "DIR_WEST", "D": "DIR_DOWN", "U": "DIR_UP"}


def build_case(ibm, case, tol=1e-12):
    m = case["meta"]
    s = ibm.IBMSolver()
    s.set_grid(case["xf"], case["yf"], case["zf"])
    s.set_params(m["re"], m["dt"])
    s.set_ext_force(*m["force"])
    if "smag" in m:
        s.set_turb_model(ibm.TURBMODEL_SMAGORINSKY, m["smag"])
    for b in m["bc"]:
        t = b.split()
        s.set_bc(getattr(ibm, _DIR[t[0]]), getattr(ibm, _BC[t[1]]), *[float(v) for v in t[2:]])
    for b in m.get("bcfunc", []):                 # VAL_FUNC faces
        face, kind, fn = b.split()
        s.set_bc(getattr(ibm, _DIR[face]), getattr(ibm, _BC[kind]), *valfuncs.BC_FUNCS[fn])
    if "forcefunc" in m:
        s.set_ext_force(*valfuncs.FORCE_FUNCS[m["forcefunc"]])
    if "stl" in m or "stl_gen" in m:
        s.set_obstacle(ibm.Polyhedron(case_stl(m)))
    s.set_linear_solver(ibm.SOLVER_BiCGSTAB, ibm.PRECOND_AMG, tol)
    s.assemble()
    s.init_flow_array(case["u1_0"], case["u2_0"], case["u3_0"], case["p_0"])
    return s


def _same_nan(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b))


@pytest.mark.parametrize("name", golden_cases())
def test_setup_bit_exact(ibm, name):
    case = load_golden(name)
    s = build_case(ibm, case)
    assert np.array_equal(s.get_flag(), case["flag"])
    lv = s.get_field("lvset")
    assert np.array_equal(lv, case["lvset"], equal_nan=True), \
        f"lvset differs at {int((lv != case['lvset']).sum())} points"
    assert np.array_equal(s.get_field("coeffsum"), case["coeffsum"])
    ijk, idx, coeff = s.ghost_stencils()
    gi = case["ghost_idx"]
    assert len(ijk) == len(gi)
    if len(gi):
        assert np.array_equal(ijk, gi[:, :3])
        assert np.array_equal(idx.reshape(len(gi), 24), gi[:, 3:])
        assert np.array_equal(coeff, case["ghost_coeff"])


_MODES = {"fp64": "FP64", "mixed": "MIXED", "mixed_mg": "MIXED_MG"}


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_mg"])
@pytest.mark.parametrize("name", golden_cases())
def test_steps_match_reference(ibm, name, precision):
    case = load_golden(name)
    s = build_case(ibm, case, tol=case["meta"].get("solve_tol", 1e-12))
    s.set_precision(getattr(ibm, _MODES[precision]))
    calls = case["meta"]["calls"]
    report = []
    for c, n in enumerate(calls, start=1):
        s.iterate(n)
        names = ["u1", "u2", "u3", "p", "U1", "U2", "U3"]
        if c == len(calls):
            names += ["u1star", "u2star", "u3star", "U1star", "U2star", "U3star", "pprime", "N1", "N2", "N3"]
        for f in names:
            got, ref = s.get_field(f), case[f"{f}_{c}"]
            assert got.shape == ref.shape, f
            assert _same_nan(got, ref), f"{f} after call {c}: NaN mask differs"
            err = rel_l2(got, ref)
            report.append((c, f, err))
            tol = PPRIME_TOL if f == "pprime" else FIELD_TOL
            assert err <= tol, f"{f} after call {c}: rel L2 {err:.3e} > {tol}"
    st = s.stats()
    assert st["iter"] == sum(calls)
    if precision == "mixed":
        assert st["outer_p"] >= 1


@pytest.mark.parametrize("precision", ["fp64", "mixed_mg"])
@pytest.mark.parametrize("name", ["sphere", "mixed_box", "func_sphere"])
def test_gmres_steps_match_reference(ibm, name, precision):
    """SOLVER_GMRES pressure solves (flexible GMRES, restart 10 as the
    reference's KDim) reach the same fields as the reference's fixtures,
    which hypre's BiCGSTAB produced: both solve to 1e-12."""
    case = load_golden(name)
    s = build_case(ibm, case)
    s.set_linear_solver(ibm.SOLVER_GMRES, ibm.PRECOND_AMG, 1e-12)
    s.set_precision(getattr(ibm, _MODES[precision]))
    calls = case["meta"]["calls"]
    for c, n in enumerate(calls, start=1):
        s.iterate(n)
        for f in ("u1", "u2", "u3", "p", "U1"):
            got, ref = s.get_field(f), case[f"{f}_{c}"]
            assert _same_nan(got, ref), f"{f} after call {c}: NaN mask differs"
            err = rel_l2(got, ref)
            assert err <= FIELD_TOL, f"{f} after call {c}: rel L2 {err:.3e}"
    assert s.stats()["outer_p"] >= 1          # GMRES cycles


@pytest.mark.parametrize("precision", ["mixed", "mixed_mg"])
@pytest.mark.parametrize("name", ["sphere", "channel_les", "func_box"])
def test_mixed_without_warm_start_matches_reference(ibm, name, precision):
    """The mixed modes start the momentum solve from u^n and the pressure
    solve from the last increment by default; started from zero (as the
    reference) they reach the same fields."""
    case = load_golden(name)
    s = build_case(ibm, case, tol=case["meta"].get("solve_tol", 1e-12))
    s.set_precision(getattr(ibm, _MODES[precision]))
    s.set_warm_start(False)
    for c, n in enumerate(case["meta"]["calls"], start=1):
        s.iterate(n)
        for f in ("u1", "u2", "u3", "p", "U1"):
            got, ref = s.get_field(f), case[f"{f}_{c}"]
            assert _same_nan(got, ref), f"{f} after call {c}: NaN mask differs"
            assert rel_l2(got, ref) <= FIELD_TOL, f"{f} after call {c}: rel L2 {rel_l2(got, ref):.3e}"
