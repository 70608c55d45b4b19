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


@pytest.mark.parametrize("precision", ["FP64", "MIXED_MG", "MIXED", "MIXED32"])
def test_exact_resume_from_state_file(ibm, tmp_path, precision):
    """The mixed modes' warm starts read the last pressure increment: it is
    part of the state, so a resumed run still continues bit for bit (the
    FP32-stage step's momentum increment starts from zero in every step)."""
    case = load_golden("sphere")
    a = build_case(ibm, case, tol=1e-8)
    a.set_precision(getattr(ibm, precision))
    a.iterate(2)
    base = str(tmp_path / "ck")
    a.export_result(base)
    b = build_case(ibm, case, tol=1e-8)
    b.set_precision(getattr(ibm, precision))
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


def test_lvset_flag_file(ibm, tmp_path):
    """src/ibm3d_export.c:262-435: level set (float) and flags (int) as
    [z][y][x] over the padded grid, with the cell-centre coordinates."""
    case = load_golden("sphere")
    s = build_case(ibm, case, tol=1e-8)
    base = str(tmp_path / "geom")
    s.export_lvset_flag(base)
    f = _read_plain(base + ".nc")
    nx, ny, nz = s.shape
    assert f["_dims"] == {"x": nx + 4, "y": ny + 4, "z": nz + 4}
    assert np.array_equal(f["lvset"], oexp.to_file_layout(s.get_field("lvset")), equal_nan=True)
    assert np.array_equal(f["flag"], np.ascontiguousarray(s.get_flag().transpose(2, 1, 0)))
    assert np.array_equal(f["flag"], np.ascontiguousarray(case["flag"].transpose(2, 1, 0)))


def test_intermediate_file(ibm, tmp_path):
    """src/ibm3d_export.c:437-650: the last step's u*, u~ and p' as float
    [time][z][y][x]; u~ = u* + dt (p(+1) - p(-1)) / (c(+1) - c(-1)) with the
    step's starting pressure on [-1, N] (src/ibm3d_fracstep.c:388-412).  The
    starting pressure is p after the previous call with its outer and ghost
    values refreshed at the start of this call (src/ibm3d_fracstep.c:45-48);
    the state file holds it as the second pressure buffer."""
    case = load_golden("sphere")
    s = build_case(ibm, case, tol=1e-8)
    s.iterate(1)
    p_prev = s.get_field("p")
    s.iterate(1)
    base = str(tmp_path / "mid")
    s.export_intermediate(base)
    s.export_result(str(tmp_path / "state"))
    f = _read_plain(base + ".nc")
    assert int(f["iter"]) == 2
    for var, fld in (("u_star", "u1star"), ("v_star", "u2star"), ("w_star", "u3star"), ("p_prime", "pprime")):
        assert np.array_equal(f[var][0], oexp.to_file_layout(s.get_field(fld)), equal_nan=True), var
    nx, ny, nz = s.shape
    shape = (nx + 4, ny + 4, nz + 4)
    n = shape[0] * shape[1] * shape[2]
    state = np.fromfile(str(tmp_path / "state.ibm3d"), dtype=np.float64, offset=40, count=26 * n).reshape((26,) + shape)
    p0 = state[13]                                           # role order: u, u_next, U, U_next, p, p_next, ...
    fluid = np.zeros(shape, dtype=bool)
    fluid[2:-2, 2:-2, 2:-2] = s.get_flag()[2:-2, 2:-2, 2:-2] == 1
    assert np.array_equal(p0[fluid], p_prev[fluid])
    dt = case["meta"]["dt"]
    coords = (f["x"], f["y"], f["z"])
    for ax, (var, fld) in enumerate((("u_tilde", "u1star"), ("v_tilde", "u2star"), ("w_tilde", "u3star"))):
        us = s.get_field(fld)
        want = np.zeros_like(us)
        sl = [slice(1, m + 3) for m in (nx, ny, nz)]         # padded indices of [-1, N]
        up, dn = list(sl), list(sl)
        up[ax] = slice(2, (nx, ny, nz)[ax] + 4)
        dn[ax] = slice(0, (nx, ny, nz)[ax] + 2)
        c = coords[ax]
        dc = c[2:] - c[:-2]
        bshape = [1, 1, 1]
        bshape[ax] = len(dc)
        want[tuple(sl)] = us[tuple(sl)] + dt * (p0[tuple(up)] - p0[tuple(dn)]) / dc.reshape(bshape)
        assert np.array_equal(f[var][0], oexp.to_file_layout(want), equal_nan=True), var


def _read_plain(path):
    sio = pytest.importorskip("scipy.io")
    with sio.netcdf_file(path, "r", mmap=False) as f:
        out = {k: np.array(v.data) for k, v in f.variables.items()}
        out["_dims"] = dict(f.dimensions)
    return out


@pytest.mark.parametrize("name", ["sphere", "channel_les", "mixed_box"])
def test_export_matches_reference_file(ibm, tmp_path, name):
    """The reference's own result file (tests/golden/configs/export_<case>:
    what its IBMSolver_export_result wrote after the case's calls, recorded
    by the netCDF stand-in): from the same FP64 fields, the library's file
    holds the same coordinates and the same float u, v, w, p, vorticity and
    Q, bit for bit."""
    ref = np.load(os.path.join(ROOT, "tests", "golden", "configs", f"export_{name}.npz"))
    case = load_golden(name)
    s = build_case(ibm, case)
    s.init_flow_array(*(ref["state_" + f] for f in FIELDS))
    base = str(tmp_path / "res")
    s.export_result(base)
    f = _read(base + ".nc")
    for var in ("x", "y", "z"):
        assert np.array_equal(f[var], ref[var]), var
    for var in ("u", "v", "w", "p", "vorticity", "Q"):
        got = f[var][0]
        assert got.dtype.kind == "f" and got.dtype.itemsize == 4 and got.shape == ref[var].shape, var
        got = got.astype("<f4")            # the file is big-endian
        assert np.array_equal(got, ref[var], equal_nan=True), \
            f"{var}: {int((got != ref[var]).sum())} values differ from the reference's file"
        # Bit for bit where finite (NaN payloads aside).
        fin = np.isfinite(ref[var])
        assert np.array_equal(got[fin].view(np.uint32), ref[var][fin].view(np.uint32)), var
