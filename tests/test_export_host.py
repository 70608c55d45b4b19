"""Host-side checks of the result export (no GPU).

* The export oracle (oracle/export_oracle.py, the restatement of
  src/ibm3d_export.c:110-141) against known answers: a linear velocity
  field on a non-uniform grid of integer coordinates, where every clamped
  central difference, the vorticity and Q are exact.
* The library's netCDF classic writer and reader (csrc/ncfile.cpp),
  compiled with a small driver, against scipy's independent reader.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import export_oracle as oexp  # noqa: E402

CSRC = os.path.join(ROOT, "2020researchproject_gb300", "csrc")


def _coords(n):
    i = np.arange(n, dtype=np.float64)
    return i * (i + 1) / 2          # integers, non-uniform spacing


def test_vorticity_q_known_answer():
    nx, ny, nz = 7, 5, 6
    x, y, z = _coords(nx), _coords(ny) * 2, _coords(nz) * 3
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")          # file layout [k][j][i]
    A = np.array([[2.0, 3.0, -1.0],                          # du/dx, du/dy, du/dz
                  [1.0, -2.0, 4.0],
                  [-3.0, 5.0, 0.0]])
    u = (A[0, 0] * X + A[0, 1] * Y + A[0, 2] * Z).astype(np.float32)
    v = (A[1, 0] * X + A[1, 1] * Y + A[1, 2] * Z).astype(np.float32)
    w = (A[2, 0] * X + A[2, 1] * Y + A[2, 2] * Z).astype(np.float32)
    vort, q = oexp.vorticity_q(u, v, w, x, y, z)
    om = np.array([A[2, 1] - A[1, 2], A[0, 2] - A[2, 0], A[1, 0] - A[0, 1]])
    qa = (A[0, 0] * A[1, 1] + A[1, 1] * A[2, 2] + A[2, 2] * A[0, 0]
          - A[0, 1] * A[1, 0] - A[1, 2] * A[2, 1] - A[0, 2] * A[2, 0])
    assert vort.dtype == np.float32 and q.dtype == np.float32
    assert np.all(vort == np.float32(np.sqrt(om @ om)))
    assert np.all(q == np.float32(qa))


def test_vorticity_q_clamps_at_the_padding():
    """A field that varies only between the first two padded cells: the
    clamped one-sided difference sees it at i = 0, the central one at i = 1."""
    n = 6
    x = np.arange(n, dtype=np.float64)
    u = np.zeros((n, n, n), np.float32)
    v = np.zeros_like(u)
    w = np.zeros_like(u)
    v[:, :, 0] = -1.0
    vort, q = oexp.vorticity_q(u, v, w, x, x, x)
    assert np.all(vort[:, :, 0] == 1.0)                       # (v1 - v0) / (x1 - x0)
    assert np.all(vort[:, :, 1] == 0.5)                       # (v2 - v0) / (x2 - x0)
    assert np.all(vort[:, :, 2:] == 0.0)
    assert np.all(q == 0.0)


def test_file_layout_transposes():
    f = np.arange(3 * 4 * 5, dtype=np.float64).reshape(3, 4, 5) + 0.1    # [i][j][k]
    g = oexp.to_file_layout(f)
    assert g.shape == (5, 4, 3) and g.dtype == np.float32
    assert g[4, 2, 1] == np.float32(f[1, 2, 4])


_DRIVER = r'''
#include "ncfile.h"
#include <cstdio>
#include <vector>
using namespace ibm;
int main(int argc, char **argv) {
    const int nx = 5, ny = 3, nz = 2;
    std::vector<double> x(nx), y(ny), z(nz);
    for (int i = 0; i < nx; i++) x[i] = 0.5 * i;
    for (int i = 0; i < ny; i++) y[i] = -1.0 + i;
    for (int i = 0; i < nz; i++) z[i] = 1e-3 * i;
    std::vector<float> u(nx * ny * nz), q(nx * ny * nz);
    for (int e = 0; e < nx * ny * nz; e++) { u[e] = 0.25f * e - 3.0f; q[e] = -1.0f / (e + 1); }
    const double t = 12.5;
    const int it = 42;
    NcFile f;
    f.dims = {{"time", 1}, {"x", nx}, {"y", ny}, {"z", nz}};
    f.vars.push_back({"time", NCT_DOUBLE, {0}, {{"axis", "T"}, {"units", "seconds"}}, &t});
    f.vars.push_back({"x", NCT_DOUBLE, {1}, {{"axis", "X"}, {"units", "meters"}}, x.data()});
    f.vars.push_back({"y", NCT_DOUBLE, {2}, {{"axis", "Y"}, {"units", "meters"}}, y.data()});
    f.vars.push_back({"z", NCT_DOUBLE, {3}, {{"axis", "Z"}, {"units", "meters"}}, z.data()});
    f.vars.push_back({"iter", NCT_INT, {}, {}, &it});
    f.vars.push_back({"u", NCT_FLOAT, {0, 3, 2, 1}, {{"units", "m/s"}}, u.data()});
    f.vars.push_back({"Q", NCT_FLOAT, {0, 3, 2, 1}, {{"units", "1/s^2"}}, q.data()});
    if (!nc_write(argv[1], f)) return 1;
    NcFile r;
    if (!nc_read_header(argv[1], r)) return 2;
    std::vector<double> a;
    for (const char *nm : {"time", "iter", "x", "u", "Q"}) {
        if (!nc_read_var(argv[1], r, nm, a)) return 3;
        printf("%s", nm);
        for (double d : a) printf(" %.17g", d);
        printf("\n");
    }
    if (nc_read_var(argv[1], r, "missing", a)) return 4;
    if (nc_read_header(argv[2], r)) return 5;    // not a netCDF file
    return 0;
}
'''


@pytest.fixture(scope="module")
def nc_driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("ncdrv")
    src = d / "drv.cpp"
    src.write_text(_DRIVER)
    exe = d / "drv"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, str(src), os.path.join(CSRC, "ncfile.cpp"),
                    "-o", str(exe)], check=True)
    return exe


def test_ncfile_round_trip_and_scipy_reader(nc_driver, tmp_path):
    path = tmp_path / "r.nc"
    junk = tmp_path / "junk.nc"
    junk.write_bytes(b"HDF\x89 not a classic netCDF file")
    out = subprocess.run([str(nc_driver), str(path), str(junk)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = {ln.split()[0]: np.array([float(v) for v in ln.split()[1:]]) for ln in out.stdout.splitlines()}
    e = np.arange(30)
    assert rows["time"].tolist() == [12.5] and rows["iter"].tolist() == [42]
    assert np.array_equal(rows["u"], (np.float32(0.25) * e.astype(np.float32) - np.float32(3)).astype(np.float64))
    assert np.array_equal(rows["Q"], (np.float32(-1) / (e + 1).astype(np.float32)).astype(np.float64))

    sio = pytest.importorskip("scipy.io")
    with sio.netcdf_file(str(path), "r", mmap=False) as f:
        assert f.version_byte == 1
        assert f.dimensions == {"time": 1, "x": 5, "y": 3, "z": 2}
        assert f.variables["time"].axis == b"T" and f.variables["time"].units == b"seconds"
        assert f.variables["x"].units == b"meters" and f.variables["z"].axis == b"Z"
        assert f.variables["u"].dimensions == ("time", "z", "y", "x")
        assert f.variables["u"].data.dtype.itemsize == 4 and f.variables["Q"].units == b"1/s^2"
        assert int(f.variables["iter"].getValue()) == 42
        assert np.array_equal(f.variables["x"].data, 0.5 * np.arange(5))
        u = np.asarray(f.variables["u"].data, dtype=np.float32)
        assert u.shape == (1, 2, 3, 5)
        assert np.array_equal(u.ravel(), np.float32(0.25) * e.astype(np.float32) - np.float32(3))


def test_restart_from_u_and_p_alone_is_not_exact_in_the_reference_algorithm():
    """Why the exact-resume file holds both buffers of every double-buffered
    field: in the reference's algorithm (restated by the oracle) a run that
    restarts from u and p alone departs from the continuing run wherever
    ghost cells exist, because update_next leaves the ghost cells of the
    next buffer at their values of two steps back and update_ghost reads
    them.  Without ghost cells u and p do suffice."""
    from conftest import load_golden
    from test_oracle_golden import oracle_case

    def run(name):
        case = load_golden(name)
        a = oracle_case(case, tol=1e-8)
        a.iterate(2)
        b = oracle_case(case, tol=1e-8)
        b.init(*(a.get(f).copy() for f in ("u1", "u2", "u3", "p")))
        a.iterate(1)
        b.iterate(1)
        return np.array_equal(a.get("u1"), b.get("u1"), equal_nan=True)

    assert run("cavity")
    assert not run("sphere")
