"""GPU parity at the benchmark configurations' full sizes.

The fixtures in tests/golden/configs/ were made by the reference itself
(tests/golden/make_config_golden.py runs the reference's own C sources):

* C2, sphere 192x128x128 around the 20,480-triangle icosphere: cell flags,
  the level set, the pressure coefficient sums and every ghost cell's
  interpolation stencil (indices and weights) must be bit-exact.  At this
  size the level set comes from the closest-point transform's full
  extrusion search, where any tie rule or rounding order that differed
  would show.
* C1, lid-driven cavity 64^3, Re 1000, dt 1e-3, 200 steps in one iterate
  call: u, v, w, p within 1e-9 relative L2 of the reference with both
  solves at relative tolerance 1e-12, in the plain FP64 step and in both
  mixed-precision forms; at the benchmark's tolerances (momentum 1e-6,
  max|div U| <= 1e-8) the mixed step's error against the reference is
  stated and bounded.
* C3, channel LES 128x96x128 (Smagorinsky, stretched walls, periodic x and
  z), 2 steps from the seeded Poiseuille-plus-noise state: the sampled
  relative L2 difference (every 4th cell along each axis) of u, v, w
  within 1e-9 and of p within 1e-7 at tolerance 1e-12 (the pressure
  starts at zero and has no boundary value: it is the sum of two
  increments p', each fixed only up to the pinned cell).
"""
import hashlib
import importlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu

CONFIGS = os.path.join(GOLDEN, "configs")
FIELD_TOL = 1e-9
# The channel's pressure has no boundary value (periodic x and z, walls in
# y): it is the sum of the increments p', each fixed only up to the pinned
# cell and solved to a residual relative to a small right-hand side; the
# velocities it drives agree to 1e-12.
PRESSURE_TOL = 1e-7
FIELDS = ("u1", "u2", "u3", "p")


def _load(name):
    z = np.load(os.path.join(CONFIGS, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["meta"] = json.loads(str(out["meta"]))
    return out


def _wl():
    return importlib.import_module("2020researchproject_gb300.workloads")


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_c2_sphere192_setup_bit_exact(ibm):
    ref = _load("c2_sphere192_setup")
    wl = _wl()
    s = wl.build_solver(ibm, wl.sphere())
    flag = s.get_flag()
    assert np.array_equal(flag.astype(np.int8), ref["flag"]), \
        f"flags differ at {int((flag.astype(np.int8) != ref['flag']).sum())} cells"
    assert _sha(flag.astype("<i4")) == ref["meta"]["flag_sha256"]
    assert _sha(s.get_field("lvset")) == ref["meta"]["lvset_sha256"], "level set not bit-exact"
    assert _sha(s.get_field("coeffsum")) == ref["meta"]["coeffsum_sha256"], "p_coeffsum not bit-exact"
    ijk, idx, coeff = s.ghost_stencils()
    gi = ref["ghost_idx"]
    assert len(ijk) == len(gi) == ref["meta"]["ghost_cells"]
    assert np.array_equal(ijk, gi[:, :3])
    assert np.array_equal(idx.reshape(len(gi), 24), gi[:, 3:])
    assert np.array_equal(coeff, ref["ghost_coeff"])
    s.close()


def _cavity(ibm, mode, tol, div_tol=0.0, warm=True):
    wl = _wl()
    case = wl.cavity(64, 1000.0, 1e-3)
    s = wl.build_solver(ibm, case, tol=tol, div_tol=div_tol)
    s.set_precision(mode)
    s.set_warm_start(warm)
    s.init_flow_array(*wl.initial_state(case))
    s.iterate(200)                       # one call, as the reference's run
    return s


@pytest.mark.parametrize("mode", ["FP64", "MIXED", "MIXED_MG"])
def test_c1_cavity64_200_steps(ibm, mode):
    ref = _load("c1_cavity64")
    s = _cavity(ibm, getattr(ibm, mode), 1e-12)
    errs = {f: rel_l2(s.get_field(f), ref[f]) for f in FIELDS}
    st = s.stats()
    s.close()
    print(mode, "errors vs the reference after 200 steps:", errs, "max|div U|", st["max_div"])
    for f, e in errs.items():
        assert e < FIELD_TOL, f"{mode} {f}: rel L2 {e:.2e} after 200 steps"
    assert st["iter"] == 200
    assert st["max_div"] < 1e-8


def test_c1_cavity64_benchmark_tolerances(ibm):
    """The benchmark's stopping rules (momentum relative residual 1e-6,
    pressure until max|div U| <= 1e-8 on fluid cells): every step meets the
    divergence bound.  After 200 steps the mixed-precision steps stay within
    1e-6 relative L2 of the reference solved to 1e-12 (their momentum solves
    start from u^n, so each step's 1e-6 residual is relative to a small
    correction); the plain FP64 step, whose momentum solves start from zero
    as the reference's do, carries the 1e-6 stopping tolerance of each of
    the 200 solves (measured 1.4e-5; bound 1e-4)."""
    ref = _load("c1_cavity64")
    out = {}
    for mode in ("FP64", "MIXED_MG", "MIXED", "MIXED32"):
        s = _cavity(ibm, getattr(ibm, mode), 1e-6, div_tol=1e-8)
        num = sum(np.sum((s.get_field(f) - ref[f]) ** 2) for f in FIELDS[:3])
        den = sum(np.sum(ref[f] ** 2) for f in FIELDS[:3])
        out[mode] = (float(np.sqrt(num / den)), s.stats()["max_div"])
        s.close()
    print("velocity rel L2 vs the reference (tol 1e-12) and max|div U|:", out)
    for mode, (err, div) in out.items():
        assert div <= 1e-8, f"{mode}: max|div U| {div:.2e}"
        bound = 1e-4 if mode == "FP64" else 1e-6
        assert err <= bound, f"{mode}: velocity rel L2 {err:.2e} vs the reference"


def test_c3_channel_les_short_horizon(ibm):
    ref = _load("c3_channel_2steps")
    wl = _wl()
    case = wl.channel()
    sample = (slice(3, -2, 4),) * 3
    for mode in ("FP64", "MIXED_MG"):
        s = wl.build_solver(ibm, case, tol=1e-12)
        s.set_precision(getattr(ibm, mode))
        s.init_flow_array(*wl.initial_state(case))
        s.iterate(2)
        errs = {f: rel_l2(s.get_field(f)[sample], ref[f]) for f in FIELDS}
        s.close()
        print(mode, "sampled errors vs the reference after 2 steps:", errs)
        for f, e in errs.items():
            # p is the sum of the two steps' increments here (p starts at 0),
            # so it carries p' tolerance.
            tol = PRESSURE_TOL if f == "p" else FIELD_TOL
            assert e < tol, f"{mode} {f}: sampled rel L2 {e:.2e}"
