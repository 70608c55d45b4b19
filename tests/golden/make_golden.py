"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference solver's own C sources (built by ``make -C oracle ref``
into oracle/_ref/ref_driver against single-rank MPI / GTree / hypre /
netCDF stand-ins) on small seeded cases and stores inputs and outputs as
.npz files.  Needs the reference tree, so it runs only where that is
mounted; the fixtures it writes are committed and travel with the tests.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import importlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
geometry = importlib.import_module("2020researchproject_gb300.geometry")

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def _stl(name, verts, faces):
    path = os.path.join(HERE, name)
    geometry.write_stl(path, verts, faces)
    return path


def _generated(gen):
    """A mesh too large to commit, written to the temporary directory."""
    path = os.path.join(tempfile.gettempdir(), f"ibm3d_golden_{gen}.stl")
    geometry.write_stl(path, *geometry.bumpy_sphere(int(gen[5:])))
    return path


def cases():
    """Small cases that together put every boundary-condition type on every
    axis, a sphere and a box body, LES on periodic and wall boundaries,
    stretched grids, split iterate() calls and time-dependent (VAL_FUNC)
    boundary values and body force."""
    sphere2 = _stl("sphere_sub2.stl", *geometry.icosphere(2, 0.5))
    sphere1 = _stl("sphere_sub1_off.stl", *geometry.icosphere(1, 0.45, (0.3, -0.2, 0.1)))
    box = _stl("box.stl", *geometry.box_union([((-0.45, -0.35, -0.3), (0.35, 0.3, 0.25))]))
    gf = geometry
    return {
        # All six faces BC_VELOCITY_COMPONENT (walls + lid), stretched grid.
        "cavity": dict(
            grid=(12, 10, 8),
            xf=gf.body_clustered_faces(0, 1, 12, 0.5, 0.5, 1.5),
            yf=gf.uniform_faces(0, 1, 10), zf=gf.body_clustered_faces(0, 1, 8, 1.0, 0.6, 1.0),
            re=100, dt=0.01, calls=[3, 2],
            bc=["W wall", "E wall", "S wall", "N wall", "D wall", "U vel 1 0 0"],
            init="field"),
        # Sphere: W velocity inflow, E pressure, slip sides (src/main.c:138-140).
        "sphere": dict(
            grid=(18, 14, 14),
            xf=gf.body_clustered_faces(-1.6, 2.4, 18, 0.0, 1.2, 1.5),
            yf=gf.body_clustered_faces(-1.4, 1.4, 14, 0.0, 1.2, 1.5),
            zf=gf.body_clustered_faces(-1.4, 1.4, 14, 0.0, 1.2, 1.5),
            re=50, dt=0.02, calls=[2, 1],
            bc=["W vel 1 0 0", "E press 0", "S slip", "N slip", "D slip", "U slip"],
            stl=sphere2, init="const 1 0 0 0"),
        # Channel LES: periodic x and z, walls in y, tanh stretching, body force.
        "channel_les": dict(
            grid=(10, 12, 8),
            xf=gf.uniform_faces(0, 2 * np.pi, 10), yf=gf.tanh_faces(12, 2.0),
            zf=gf.uniform_faces(0, np.pi, 8),
            re=400, dt=0.01, calls=[3], force=(2 / 400, 0, 0), smag=0.1,
            bc=["W per", "E per", "S wall", "N wall", "D per", "U per"],
            init="field"),
        # Pressure on W/D/U, velocity on E, velocity-periodic S/N, box body.
        "mixed_box": dict(
            grid=(14, 12, 10),
            xf=gf.uniform_faces(-1.2, 1.6, 14), yf=gf.body_clustered_faces(-1.0, 1.0, 12, 0, 0.7, 1.0),
            zf=gf.uniform_faces(-0.9, 1.1, 10),
            re=80, dt=0.01, calls=[2],
            bc=["W press 0.2", "E vel -0.3 0.1 0", "S velper 0", "N velper 0", "D press 0", "U press 0.1"],
            stl=box, init="field"),
        # Slip W/E, velocity S, pressure N, velocity-periodic D/U, offset sphere.
        "mixed_sphere": dict(
            grid=(14, 14, 12),
            xf=gf.uniform_faces(-1.0, 1.6, 14), yf=gf.uniform_faces(-1.3, 1.2, 14),
            zf=gf.body_clustered_faces(-1.0, 1.2, 12, 0.1, 0.8, 1.0),
            re=60, dt=0.01, calls=[1, 1],
            bc=["W slip", "E slip", "S vel 0.1 0.4 0", "N press 0", "D velper 0.05", "U velper 0.05"],
            stl=sphere1, init="field"),
        # VAL_FUNC: time-dependent inflow on W, time-dependent outlet
        # pressure on E, slip sides, time-dependent body force, sphere
        # (src/ibm3d_fracstep.c:1978-2035); split call so time carries on.
        "func_sphere": dict(
            grid=(16, 12, 12),
            xf=gf.body_clustered_faces(-1.6, 2.4, 16, 0.0, 1.2, 1.5),
            yf=gf.body_clustered_faces(-1.4, 1.4, 12, 0.0, 1.2, 1.5),
            zf=gf.body_clustered_faces(-1.4, 1.4, 12, 0.0, 1.2, 1.5),
            re=50, dt=0.02, calls=[2, 2],
            bc=["S slip", "N slip", "D slip", "U slip"],
            bcfunc=["W vel pulse", "E press ramp"], forcefunc="swirl",
            stl=sphere2, init="const 1 0 0 0"),
        # VAL_FUNC on velocity-periodic x (pressure jump in time), velocity
        # D and pressure U, walls S/N, box body, constant force.
        "func_box": dict(
            grid=(12, 10, 12),
            xf=gf.uniform_faces(-1.2, 1.6, 12), yf=gf.body_clustered_faces(-1.0, 1.0, 10, 0, 0.7, 1.0),
            zf=gf.uniform_faces(-0.9, 1.1, 12),
            re=80, dt=0.01, calls=[3], force=(0.01, 0, 0),
            bc=["S wall", "N wall"],
            bcfunc=["W velper ramp", "E velper ramp", "D vel pulse", "U press ramp"],
            stl=box, init="field"),
        # A large body: 81,920 triangles with dents and bulges (the mesh is
        # regenerated by the tests, not committed), W inflow, E outlet.
        "bumpy_stl": dict(
            grid=(40, 36, 36),
            xf=gf.body_clustered_faces(-1.2, 1.6, 40, 0.0, 0.8, 1.5),
            yf=gf.body_clustered_faces(-1.0, 1.0, 36, 0.0, 0.8, 1.5),
            zf=gf.body_clustered_faces(-1.0, 1.0, 36, 0.0, 0.8, 1.5),
            re=100, dt=0.01, calls=[1],
            bc=["W vel 1 0 0", "E press 0", "S slip", "N slip", "D slip", "U slip"],
            stl=_generated("bumpy6"), stl_gen="bumpy6", init="const 1 0 0 0",
            # The first step from uniform flow past a large body has a steep
            # pressure: a relative residual of 1e-12 still leaves 1e-8 in the
            # fields, so the parity tests solve to 1e-14 (the reference's
            # solve landed within 1e-11 of that).
            solve_tol=1e-14),
        # Velocity-periodic x, all-periodic y, velocity D, pressure U, LES.
        "mixed_les": dict(
            grid=(10, 8, 12),
            xf=gf.uniform_faces(0, 2.0, 10), yf=gf.uniform_faces(0, 1.5, 8),
            zf=gf.tanh_faces(12, 1.5, 0.0, 1.0),
            re=300, dt=0.01, calls=[2], smag=0.15,
            bc=["W velper 0", "E velper 0", "S per", "N per", "D vel 0.2 0 0", "U press 0"],
            init="field"),
    }


def write_case_file(path, c):
    nx, ny, nz = c["grid"]
    with open(path, "w") as fh:
        fh.write(f"grid {nx} {ny} {nz}\n")
        for key in ("xf", "yf", "zf"):
            fh.write(key + " " + " ".join(repr(float(v)) for v in c[key]) + "\n")
        fh.write(f"re {c['re']!r}\ndt {c['dt']!r}\ntol 1e-12\n")
        fh.write("calls " + " ".join(str(n) for n in c["calls"]) + "\n")
        for b in c["bc"]:
            fh.write("bc " + b + "\n")
        for b in c.get("bcfunc", []):
            fh.write("bcfunc " + b + "\n")
        if "forcefunc" in c:
            fh.write(f"forcefunc {c['forcefunc']}\n")
        if "force" in c:
            fh.write("force %r %r %r\n" % tuple(float(v) for v in c["force"]))
        if "smag" in c:
            fh.write(f"smag {c['smag']!r}\n")
        if "stl" in c:
            fh.write(f"stl {c['stl']}\n")
        fh.write(f"init {c['init']}\n")


def run_case(name, c):
    nx, ny, nz = c["grid"]
    cell = (nx + 4, ny + 4, nz + 4)
    shapes = {"U1": (nx + 1, ny + 4, nz + 4), "U2": (nx + 4, ny + 1, nz + 4), "U3": (nx + 4, ny + 4, nz + 1)}
    with tempfile.TemporaryDirectory() as tmp:
        cf = os.path.join(tmp, "case.txt")
        write_case_file(cf, c)
        subprocess.run([DRIVER, cf, tmp], check=True)
        out = {}

        def load(fname, dtype, shape):
            return np.fromfile(os.path.join(tmp, fname), dtype=dtype).reshape(shape)

        out["flag"] = load("flag.i32", "<i4", cell)
        out["lvset"] = load("lvset.f64", "<f8", cell)
        out["coeffsum"] = load("coeffsum.f64", "<f8", cell)
        g = []
        with open(os.path.join(tmp, "ghost.txt")) as fh:
            for line in fh:
                t = line.split()
                g.append([int(v) for v in t[:27]] + [float.fromhex(v) for v in t[27:]])
        out["ghost_idx"] = np.array([r[:27] for r in g], dtype=np.int32).reshape(-1, 27)
        out["ghost_coeff"] = np.array([r[27:] for r in g], dtype=np.float64).reshape(-1, 8)
        for f in ("u1", "u2", "u3", "p"):
            out[f + "_0"] = load(f + "_0.f64", "<f8", cell)
        ncalls = len(c["calls"])
        for s in range(1, ncalls + 1):
            names = ["u1", "u2", "u3", "p", "U1", "U2", "U3"]
            if s == ncalls:
                names += ["u1star", "u2star", "u3star", "U1star", "U2star", "U3star", "pprime", "N1", "N2", "N3"]
            for f in names:
                base = f[:2] if f.startswith("U") else None
                shape = shapes.get(base, cell)
                out[f"{f}_{s}"] = load(f"{f}_{s}.f64", "<f8", shape)
        meta = dict(c)
        meta.pop("xf"), meta.pop("yf"), meta.pop("zf")
        if "stl_gen" in meta:
            meta.pop("stl")
        elif "stl" in meta:
            meta["stl"] = os.path.basename(meta["stl"])
        meta["force"] = list(meta.get("force", (0, 0, 0)))
        out["meta"] = np.array(json.dumps(meta))
        out["xf"], out["yf"], out["zf"] = (np.asarray(c[k], dtype=np.float64) for k in ("xf", "yf", "zf"))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: {len(out['ghost_idx'])} ghost cells, "
              f"{int((out['flag'] == 3).sum())} solid, calls {c['calls']}")


def main(argv):
    if not os.path.exists(DRIVER):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    all_cases = cases()
    for name in argv or list(all_cases):
        run_case(name, all_cases[name])


if __name__ == "__main__":
    main(sys.argv[1:])
