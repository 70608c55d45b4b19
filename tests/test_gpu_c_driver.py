"""The C case driver (tests/drivers/ibm3d_driver.c) run on the GPU: it
calls only the public C API (variadic set_bc / set_ext_force /
set_turb_model, an STL obstacle through fopen_check, iterate with the
per-step log, export_result) and its fields after a few steps must match
the CPU oracle on the same case: velocity within 1e-9 relative L2,
pressure within 1e-8 (both solve to tolerance 1e-12; the pressure carries
the Poisson solve's conditioning, as p' does in the golden tests)."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

from c_driver import build_driver
from conftest import GOLDEN, ROOT, rel_l2

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def _faces(n, lo, hi):
    return np.array([lo + (hi - lo) * i / n for i in range(n + 1)])


def _case(kind, n):
    if kind == "cavity":
        f = _faces(n, 0.0, 1.0)
        return dict(xf=f, yf=f, zf=f, re=400.0, dt=2e-3, u0=0.0,
                    bc=["U vel 1 0 0", "W wall", "E wall", "S wall", "N wall", "D wall"])
    if kind == "channel":
        yf = np.array([math.tanh(2.0 * (2.0 * j / n - 1)) / math.tanh(2.0) for j in range(n + 1)])
        return dict(xf=_faces(n, 0.0, 2 * math.pi), yf=yf, zf=_faces(n, 0.0, math.pi), re=3000.0, dt=5e-3, u0=1.0,
                    force=(2.0 / 3000.0, 0.0, 0.0), smag=0.1,
                    bc=["W per", "E per", "D per", "U per", "S wall", "N wall"])
    return dict(xf=_faces(n, -1.5, 2.5), yf=_faces(n, -1.5, 1.5), zf=_faces(n, -1.5, 1.5), re=100.0, dt=1e-2,
                u0=1.0, stl=os.path.join(GOLDEN, "sphere_sub2.stl"),
                bc=["W vel 1 0 0", "E press 0", "N slip", "S slip", "D slip", "U slip"])


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    return build_driver(tmp_path_factory.mktemp("driver"))


@pytest.mark.parametrize("kind,n,steps", [("cavity", 16, 5), ("channel", 16, 4), ("sphere", 20, 3)])
def test_c_driver_matches_oracle(driver, tmp_path, kind, n, steps):
    import oracle as orc
    c = _case(kind, n)
    out = os.path.join(str(tmp_path), kind)
    args = [driver, kind, str(n), str(steps), out] + ([c["stl"]] if "stl" in c else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    # The per-step log: the reference's columns plus max|div U|.
    assert "max|div U|" in r.stdout
    rows = [ln.split() for ln in r.stdout.splitlines() if ln.strip()[:1].isdigit() and len(ln.split()) == 7]
    assert [int(t[0]) for t in rows] == list(range(1, steps + 1))
    assert all(float(t[6]) < 1e-8 for t in rows)
    assert os.path.exists(out + ".nc") and os.path.exists(out + ".ibm3d")

    shape = (n + 4,) * 3
    got = {f: np.fromfile(f"{out}_{f}.f64", dtype="<f8").reshape(shape) for f in ("u1", "u2", "u3", "p")}
    oc = {k: v for k, v in c.items() if k != "u0"}
    oc.update(tol=1e-12, threads=os.cpu_count() or 1)
    o = orc.Oracle(oc)
    o.init(np.full(shape, c["u0"]), np.zeros(shape), np.zeros(shape), np.zeros(shape))
    o.iterate(steps)
    ref = {f: o.get(f) for f in ("u1", "u2", "u3", "p")}
    for f in ref:
        assert np.array_equal(np.isnan(got[f]), np.isnan(ref[f])), f"{kind} {f}: NaN masks differ"
    # Velocity as one vector field (a component that stays near zero, as
    # the spanwise one of the channel, has no scale of its own), p alone.
    m = np.isfinite(ref["u1"])
    num = sum(np.sum((got[f][m] - ref[f][m]) ** 2) for f in ("u1", "u2", "u3"))
    den = sum(np.sum(ref[f][m] ** 2) for f in ("u1", "u2", "u3"))
    err_u = float(np.sqrt(num / den))
    err_p = rel_l2(got["p"], ref["p"])
    assert err_u < 1e-9, f"{kind} velocity: rel L2 {err_u:.2e} vs the oracle"
    assert err_p < 1e-8, f"{kind} p: rel L2 {err_p:.2e} vs the oracle"
