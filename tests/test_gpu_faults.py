"""Failure detection in the time step, with the failure made on the host
(no GPU fault): an iteration cap too small for the tolerance, and NaN in
the host initial-state buffer.

* A solve that reaches its cap prints the reference's warning and the step
  continues (src/ibm3d_fracstep.c:363-369, 673-679).
* NaN in the state reaches the solves as non-finite dot products: the
  device ends each solve at once (a breakdown, not a run to the cap) and
  the iterate call stops after that step with IBM3D_ENONFINITE, where the
  reference would carry the NaN on silently.
"""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_golden import build_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["FP64", "MIXED"])
def test_iteration_cap_warns_and_continues(ibm, capfd, mode):
    case = load_golden("sphere")
    s = build_case(ibm, case)
    s.set_precision(getattr(ibm, mode))
    s.set_max_iters(1, 1)
    s.set_refinement(5e-7, 1e-5, 1)                # mixed: one refinement cycle
    s.iterate(2)                                   # no exception: warnings only
    err = capfd.readouterr().err
    assert "warning: p_prime did not converge" in err
    assert "did not converge" in err.replace("p_prime", "")
    st = s.stats()
    assert st["iter"] == 2 and st["iters_p"] <= 1
    for f in ("u1", "u2", "u3", "p"):
        v = s.get_field(f)
        assert np.isfinite(v[s.get_flag() == 1]).all()
    s.set_max_iters(200, 1000)                     # back to the reference's caps: converges again
    s.set_refinement(5e-7, 1e-5, 12)
    s.iterate(1)
    st = s.stats()
    assert st["res_p"] < 1e-12 and st["iter"] == 3


@pytest.mark.parametrize("mode,graphs", [("FP64", True), ("MIXED", True), ("FP64", False)])
def test_nan_in_initial_state_gives_status(ibm, mode, graphs):
    case = load_golden("sphere")
    s = build_case(ibm, case)
    s.set_precision(getattr(ibm, mode))
    s.set_graphs(graphs)
    u1 = case["u1_0"].copy()
    flag = s.get_flag()
    fl = np.argwhere(flag == 1)
    i, j, k = fl[len(fl) // 2]
    u1[i, j, k] = np.nan                           # one fluid cell of the host buffer
    s.init_flow_array(u1, case["u2_0"], case["u3_0"], case["p_0"])
    with pytest.raises(ibm.IBM3DError, match="non-finite"):
        s.iterate(5)
    st = s.stats()
    assert st["iter"] == 1                         # stopped after the first step
    assert st["iters_p"] < 50 and max(st["iters_u"]) < 50   # ended early, not at the caps (1000, 200)
    s.close()
    # The device stays usable: a new solver on a clean state steps normally.
    s2 = build_case(ibm, case)
    s2.set_precision(getattr(ibm, mode))
    s2.iterate(1)
    assert s2.stats()["res_p"] < 1e-12
