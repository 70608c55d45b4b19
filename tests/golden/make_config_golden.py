"""Golden fixtures at the benchmark configurations' full sizes, made by the
reference itself (oracle/_ref/ref_driver: the reference's own C sources
against the single-rank stand-ins, see oracle/Makefile).

Written to tests/golden/configs/:

* ``c1_cavity64.npz`` - lid-driven cavity, uniform 64^3 grid on the unit
  cube, Re 1000, dt 1e-3, lid u = 1 on the top face, walls elsewhere, fluid
  at rest, 200 steps (the reference's src/cavity.c set-up at this size), both
  linear solves to relative tolerance 1e-12.  Stores u1, u2, u3, p after the
  200 steps (padded layout) and the largest |div U| over fluid cells.
* ``c2_sphere192_setup.npz`` - the 192x128x128 body-clustered sphere grid
  around the 20,480-triangle icosphere (r = 0.5): the reference's cell
  flags (int8, compressed), SHA-256 digests of its level set and pressure
  coefficient sums (27 MB each, so only their digests are stored: the
  comparison is bit-exact), and every ghost cell's interpolation stencil
  (indices and weights) from IBMSolver_ghost_interp.
* ``c3_channel_2steps.npz`` - channel LES 2pi x 2 x pi, 128x96x128 cells,
  tanh-stretched walls (beta 2), periodic x and z, Smagorinsky Cs 0.1,
  body force 2/Re with Re 16200 (Re_tau 180), dt 2e-3, from the seeded
  Poiseuille-plus-noise state of workloads.initial_state, 2 steps at
  relative tolerance 1e-12.  The fields are 14 MB each, so the fixture
  keeps every 4th interior cell along each axis (a regular sample of
  24,576 cells) of u1, u2, u3 and p: a sampled relative L2 difference.

* ``export_<case>.npz`` for the golden cases sphere, channel_les and
  mixed_box - the reference's result file: what its IBMSolver_export_result
  hands to netCDF after the case's calls (the stand-in records every
  variable, see oracle/ref_shim): x, y, z, time, iter and the float u, v,
  w, p, vorticity and Q in [z][y][x] order, beside the FP64 fields it was
  made from (u1, u2, u3, p, padded layout).

Needs the reference tree (see oracle/Makefile), so it runs where that is
mounted; the fixtures are committed.

    python tests/golden/make_config_golden.py [c1] [c2] [c3] [exports]
"""
from __future__ import annotations

import hashlib
import importlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "configs")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
wl = importlib.import_module("2020researchproject_gb300.workloads")
from make_golden import DRIVER, write_case_file  # noqa: E402


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _run(c, tmp):
    cf = os.path.join(tmp, "case.txt")
    write_case_file(cf, c)
    t0 = time.perf_counter()
    subprocess.run([DRIVER, cf, tmp], check=True)
    return time.perf_counter() - t0


def _ghosts(tmp):
    g = []
    with open(os.path.join(tmp, "ghost.txt")) as fh:
        for line in fh:
            t = line.split()
            g.append([int(v) for v in t[:27]] + [float.fromhex(v) for v in t[27:]])
    idx = np.array([r[:27] for r in g], dtype=np.int32).reshape(-1, 27)
    coeff = np.array([r[27:] for r in g], dtype=np.float64).reshape(-1, 8)
    return idx, coeff


def max_div_fluid(case, U1, U2, U3, flag):
    """max |div U| over fluid cells from the face velocities in the
    reference's staggered layouts (U1 (nx+1, ny+4, nz+4), ...)."""
    xf, yf, zf = (np.asarray(case[k]) for k in ("xf", "yf", "zf"))
    dx, dy, dz = np.diff(xf), np.diff(yf), np.diff(zf)
    u = U1[:, 2:-2, 2:-2]
    v = U2[2:-2, :, 2:-2]
    w = U3[2:-2, 2:-2, :]
    div = ((u[1:] - u[:-1]) / dx[:, None, None] + (v[:, 1:] - v[:, :-1]) / dy[None, :, None]
           + (w[:, :, 1:] - w[:, :, :-1]) / dz[None, None, :])
    fl = flag[2:-2, 2:-2, 2:-2] == 1
    return float(np.abs(div[fl]).max())


def c1():
    case = wl.cavity(64, 1000.0, 1e-3)
    n = 64
    c = dict(grid=(n, n, n), xf=case["xf"], yf=case["yf"], zf=case["zf"], re=case["re"], dt=case["dt"],
             calls=[200], bc=list(case["bc"]), init="const 0 0 0 0")
    cell = (n + 4,) * 3
    with tempfile.TemporaryDirectory() as tmp:
        secs = _run(c, tmp)

        def load(name, shape):
            return np.fromfile(os.path.join(tmp, name), dtype="<f8").reshape(shape)

        out = {f: load(f"{f}_1.f64", cell) for f in ("u1", "u2", "u3", "p")}
        U1 = load("U1_1.f64", (n + 1, n + 4, n + 4))
        U2 = load("U2_1.f64", (n + 4, n + 1, n + 4))
        U3 = load("U3_1.f64", (n + 4, n + 4, n + 1))
        flag = np.fromfile(os.path.join(tmp, "flag.i32"), dtype="<i4").reshape(cell)
        meta = dict(config="cavity 64^3, Re 1000, dt 1e-3, lid u=1, 200 steps", steps=200, tol=1e-12,
                    max_div=max_div_fluid(case, U1, U2, U3, flag), reference_seconds=round(secs, 1))
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, "c1_cavity64.npz"), **out)
    print("c1:", meta)


def c2():
    case = wl.sphere()
    nx, ny, nz = (len(case[k]) - 1 for k in ("xf", "yf", "zf"))
    c = dict(grid=(nx, ny, nz), xf=case["xf"], yf=case["yf"], zf=case["zf"], re=case["re"], dt=case["dt"],
             calls=[], bc=list(case["bc"]), stl=case["stl"], init="const 1 0 0 0")
    cell = (nx + 4, ny + 4, nz + 4)
    with tempfile.TemporaryDirectory() as tmp:
        secs = _run(c, tmp)
        flag = np.fromfile(os.path.join(tmp, "flag.i32"), dtype="<i4").reshape(cell)
        lvset = np.fromfile(os.path.join(tmp, "lvset.f64"), dtype="<f8").reshape(cell)
        coeffsum = np.fromfile(os.path.join(tmp, "coeffsum.f64"), dtype="<f8").reshape(cell)
        idx, coeff = _ghosts(tmp)
    meta = dict(config="sphere 192x128x128 body-clustered grid, 20480-triangle icosphere r=0.5",
                lvset_sha256=digest(lvset), coeffsum_sha256=digest(coeffsum), flag_sha256=digest(flag),
                ghost_cells=int(len(idx)), solid_cells=int((flag == 3).sum()), reference_seconds=round(secs, 1))
    out = dict(flag=flag.astype(np.int8), ghost_idx=idx, ghost_coeff=coeff,
               lvset_nan=np.isnan(lvset), meta=np.array(json.dumps(meta)))
    np.savez_compressed(os.path.join(OUT, "c2_sphere192_setup.npz"), **out)
    print("c2:", meta)


C3_SAMPLE = (slice(3, -2, 4),) * 3       # padded index 3, 7, ... = interior 1, 5, ...


def c3():
    case = wl.channel()
    nx, ny, nz = (len(case[k]) - 1 for k in ("xf", "yf", "zf"))
    with tempfile.TemporaryDirectory() as tmp:
        for name, a in zip(("u1", "u2", "u3", "p"), wl.initial_state(case)):
            np.ascontiguousarray(a, dtype="<f8").tofile(os.path.join(tmp, name + ".f64"))
        c = dict(grid=(nx, ny, nz), xf=case["xf"], yf=case["yf"], zf=case["zf"], re=case["re"], dt=case["dt"],
                 calls=[2], bc=list(case["bc"]), force=case["force"], smag=case["smag"], init=f"raw {tmp}")
        secs = _run(c, tmp)
        cell = (nx + 4, ny + 4, nz + 4)
        out = {f: np.fromfile(os.path.join(tmp, f"{f}_1.f64"), dtype="<f8").reshape(cell)[C3_SAMPLE].copy()
               for f in ("u1", "u2", "u3", "p")}
    meta = dict(config="channel LES 128x96x128, Re 16200, Cs 0.1, dt 2e-3, 2 steps", steps=2, tol=1e-12,
                sample="padded indices 3::4 along each axis", reference_seconds=round(secs, 1))
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, "c3_channel_2steps.npz"), **out)
    print("c3:", meta)


EXPORT_CASES = ("sphere", "channel_les", "mixed_box")


def exports():
    from make_golden import cases
    all_cases = cases()
    for name in EXPORT_CASES:
        c = all_cases[name]
        nx, ny, nz = c["grid"]
        cell = (nx + 4, ny + 4, nz + 4)
        with tempfile.TemporaryDirectory() as tmp:
            cf = os.path.join(tmp, "case.txt")
            write_case_file(cf, c)
            with open(cf, "a") as fh:
                fh.write("export result\n")
            dump = os.path.join(tmp, "nc")
            os.makedirs(dump)
            subprocess.run([DRIVER, cf, tmp], check=True, env=dict(os.environ, IBM3D_NC_DUMP_DIR=dump))
            last = len(c["calls"])

            def raw(var, dtype, shape):
                return np.fromfile(os.path.join(dump, var + ".bin"), dtype=dtype).reshape(shape)

            pad = (nz + 4, ny + 4, nx + 4)
            out = {v: raw(v, "<f4", pad) for v in ("u", "v", "w", "p", "vorticity", "Q")}
            out.update(x=raw("x", "<f8", (nx + 4,)), y=raw("y", "<f8", (ny + 4,)), z=raw("z", "<f8", (nz + 4,)),
                       time=raw("time", "<f8", (1,)), iter=raw("iter", "<i4", (1,)))
            for f in ("u1", "u2", "u3", "p"):
                out["state_" + f] = np.fromfile(os.path.join(tmp, f"{f}_{last}.f64"), dtype="<f8").reshape(cell)
        out["meta"] = np.array(json.dumps(dict(case=name, calls=c["calls"])))
        np.savez_compressed(os.path.join(OUT, f"export_{name}.npz"), **out)
        print("export:", name, {k: v.shape for k, v in out.items() if k != "meta"})


if __name__ == "__main__":
    if not os.path.exists(DRIVER):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    os.makedirs(OUT, exist_ok=True)
    for name in sys.argv[1:] or ["c1", "c2", "c3", "exports"]:
        {"c1": c1, "c2": c2, "c3": c3, "exports": exports}[name]()
