"""Initial guess of the warm-started pressure solve (IBMSolver_set_pressure_guess):
the last increment p'_{n-1} (0) or the extrapolation 2 p'_{n-1} - p'_{n-2}
(1, the default).  Only the starting point differs: on the golden
fixtures both meet the same divergence bound every step and give fields
within 5e-7 (velocity) and 1e-5 (p) relative L2 of each other.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from test_gpu_golden import build_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sphere", "channel_les", "func_sphere"])
def test_guesses_meet_the_same_bound(ibm, name):
    case = load_golden(name)
    out = []
    for guess in (0, 1):
        s = build_case(ibm, case, tol=1e-7)
        s.set_div_tol(1e-10)
        s.set_precision(ibm.MIXED32)
        s.set_pressure_guess(guess)
        for n in case["meta"]["calls"]:
            s.iterate(n)
        st = s.stats()
        print(name, "guess", guess, "max|div U|", st["max_div_max"], "pressure iterations", st["iters_p_total"])
        assert st["max_div_max"] <= 1e-10
        out.append({f: s.get_field(f) for f in ("u1", "u2", "u3", "p")})
    for f in ("u1", "u2", "u3", "p"):
        assert np.array_equal(np.isnan(out[0][f]), np.isnan(out[1][f])), f
        assert rel_l2(out[1][f], out[0][f]) < (1e-5 if f == "p" else 5e-7), (f, rel_l2(out[1][f], out[0][f]))


def test_pressure_guess_argument(ibm):
    s = ibm.IBMSolver()
    with pytest.raises(ibm.IBM3DError):
        s.set_pressure_guess(2)
