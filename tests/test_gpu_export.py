"""Result export and restart through the C ABI (src/ibm3d_export.c:16-253,
src/ibm3d_init.c:45-224).

* "<name>.nc" holds the reference's variables and attributes; u, v, w, p
  are the float32 of the solver's FP64 fields in [time][z][y][x] order, and
  vorticity and Q (computed on the GPU) equal the export oracle's values
  from the file's own u, v, w and coordinates, bit for bit.
* "<name>.ibm3d" resumes exactly: a solver restarted from it continues
  bit for bit as the exporting solver does.
* Without the FP64 state the float fields, time and iter of the .nc file
  are read, as the reference reads them.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, load_golden
from test_gpu_golden import build_case

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import export_oracle as oexp  # noqa: E402

pytestmark = pytest.mark.gpu

FIELDS = ["u1", "u2", "u3", "p"]


def _read(path):
    sio = pytest.importorskip("scipy.io")
    with sio.netcdf_file(path, "r", mmap=False) as f:
        out = {k: np.array(v.data) for k, v in f.variables.items()}
        out["_dims"] = dict(f.dimensions)
        out["_units"] = {k: getattr(v, "units", b"") for k, v in f.variables.items()}
        out["_iter"] = int(f.variables["iter"].getValue())
    return out


@pytest.mark.parametrize("name", ["sphere", "channel_les"])
def test_export_matches_oracle(ibm, tmp_path, name):
    case = load_golden(name)
    s = build_case(ibm, case, tol=1e-8)
    s.iterate(2)
    base = str(tmp_path / "res")
    s.export_result(base)
    f = _read(base + ".nc")
    nx, ny, nz = s.shape
    assert f["_dims"] == {"time": 1, "x": nx + 4, "y": ny + 4, "z": nz + 4}
    assert f["_iter"] == 2
    assert f["time"].tolist() == [s.stats()["time"]]
    assert f["_units"]["u"] == b"m/s" and f["_units"]["vorticity"] == b"1/s" and f["_units"]["Q"] == b"1/s^2"
    xc = 0.5 * (case["xf"][1:] + case["xf"][:-1])
    assert np.array_equal(f["x"][2:-2], xc)
    for fld, var in zip(FIELDS, "uvwp"):
        got = f[var][0]
        assert got.dtype.itemsize == 4 and got.shape == (nz + 4, ny + 4, nx + 4)
        want = oexp.to_file_layout(s.get_field(fld))
        assert np.array_equal(got, want, equal_nan=True), var
    vort, q = oexp.vorticity_q(f["u"][0], f["v"][0], f["w"][0], f["x"], f["y"], f["z"])
    assert np.array_equal(f["vorticity"][0], vort, equal_nan=True)
    assert np.array_equal(f["Q"][0], q, equal_nan=True)
    assert np.isfinite(vort).sum() > 0


def test_exact_resume_from_state_file(ibm, tmp_path):
    case = load_golden("sphere")
    a = build_case(ibm, case, tol=1e-8)
    a.iterate(2)
    base = str(tmp_path / "ck")
    a.export_result(base)
    b = build_case(ibm, case, tol=1e-8)
    b.init_flow_file(base)
    assert b.stats()["iter"] == 2 and b.stats()["time"] == a.stats()["time"]
    a.iterate(2)
    b.iterate(2)
    assert b.stats()["iter"] == 4 and b.stats()["time"] == a.stats()["time"]
    for fld in FIELDS + ["U1", "pprime"]:
        assert np.array_equal(a.get_field(fld), b.get_field(fld), equal_nan=True), fld


def test_restart_from_result_file_reads_float_fields(ibm, tmp_path):
    case = load_golden("cavity")
    a = build_case(ibm, case, tol=1e-8)
    a.iterate(3)
    base = str(tmp_path / "nc_only")
    a.export_result(base)
    os.remove(base + ".ibm3d")
    b = build_case(ibm, case, tol=1e-8)
    b.init_flow_file(base)
    st = b.stats()
    assert st["iter"] == 3 and st["time"] == a.stats()["time"]
    for fld in FIELDS:
        want = a.get_field(fld).astype(np.float32).astype(np.float64)
        assert np.array_equal(b.get_field(fld), want, equal_nan=True), fld
    b.iterate(1)
    assert np.isfinite(b.get_field("u1")).any()


def test_restart_errors(ibm, tmp_path):
    case, other = load_golden("cavity"), load_golden("sphere")
    s = build_case(ibm, case, tol=1e-8)
    with pytest.raises(ibm.IBM3DError, match="cannot open"):
        s.init_flow_file(str(tmp_path / "missing"))
    t = build_case(ibm, other, tol=1e-8)
    base = str(tmp_path / "sph")
    t.export_result(base)
    with pytest.raises(ibm.IBM3DError, match="not a flow file of this grid"):
        s.init_flow_file(base)
    os.remove(base + ".ibm3d")
    with pytest.raises(ibm.IBM3DError, match="not a flow file of this grid"):
        s.init_flow_file(base)
    s.iterate(1)                      # a failed restart leaves the solver usable
