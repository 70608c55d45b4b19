"""The IBM3D_MIXED32 step: FP32 explicit stages and an FP32 momentum
solve on the increment u* - u^n, FP64 state updates, projection and
pressure Krylov (FP32 multigrid).

* Its integer-pipe FP64 <-> FP32 conversions equal the hardware's bit for
  bit (away from exact rounding ties).
* On every golden fixture made by the reference, with the momentum solved
  to 1e-7 and the pressure until max|div U| <= 1e-11 (FP64 pressure
  vectors) or 1e-10 (double-float pressure vectors, the default: their
  residual floor is ~5e-11), u, v, w and the face velocities stay within
  2e-6 relative L2 of the reference and p within 1e-5 (the FP32 rounding
  of O(dt) increments, which the pressure, a sum of increments solved
  from the velocity's divergence, amplifies; the FP64 modes match to
  1e-9).
* Recorded-graph and host-sequenced steps are bitwise identical.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_l2
from test_gpu_golden import build_case

pytestmark = pytest.mark.gpu

MIXED32_TOL = 2e-6
MIXED32_P_TOL = 1e-5


def test_conversions_match_hardware(ibm):
    rng = np.random.default_rng(7)
    vals = np.concatenate([
        rng.uniform(-2.0, 2.0, 200000),
        rng.normal(0.0, 1e3, 200000),
        10.0 ** rng.uniform(-37, 38, 200000) * rng.choice([-1.0, 1.0], 200000),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.4028234663852886e38, 1.1754943508222875e-38]),
    ])
    assert ibm.check_fp32_conversions(vals) == 0


DIV_TOL = {"fp64": 1e-11, "dfloat": 1e-10}


def _run32(ibm, case, graphs=True, pvec="dfloat"):
    s = build_case(ibm, case, tol=1e-7)
    s.set_div_tol(DIV_TOL[pvec])
    s.set_precision(ibm.MIXED32)
    s.set_pressure_vectors(ibm.PVEC_FP64 if pvec == "fp64" else ibm.PVEC_DFLOAT)
    s.set_graphs(graphs)
    for n in case["meta"]["calls"]:
        s.iterate(n)
    return s


@pytest.mark.parametrize("pvec", ["dfloat", "fp64"])
@pytest.mark.parametrize("name", golden_cases())
def test_mixed32_matches_reference(ibm, name, pvec):
    case = load_golden(name)
    s = _run32(ibm, case, pvec=pvec)
    last = len(case["meta"]["calls"])
    errs = {}
    for f in ("u1", "u2", "u3", "p", "U1", "U2", "U3"):
        got, ref = s.get_field(f), case[f"{f}_{last}"]
        assert np.array_equal(np.isnan(got), np.isnan(ref)), f"{name} {f}: NaN masks differ"
        errs[f] = rel_l2(got, ref)
    st = s.stats()
    print(name, pvec, {k: f"{v:.1e}" for k, v in errs.items()}, "max|div U|", st["max_div"])
    assert st["max_div"] <= DIV_TOL[pvec]
    for f, e in errs.items():
        assert e < (MIXED32_P_TOL if f == "p" else MIXED32_TOL), f"{name} {f}: rel L2 {e:.2e}"


@pytest.mark.parametrize("name", ["sphere", "channel_les", "func_box"])
def test_mixed32_graph_equals_host_loop(ibm, name):
    case = load_golden(name)
    a = _run32(ibm, case, graphs=True)
    b = _run32(ibm, case, graphs=False)
    for f in ("u1", "u2", "u3", "p", "U1"):
        assert np.array_equal(a.get_field(f), b.get_field(f), equal_nan=True), f
