"""Synthetic workloads of the immersed-boundary fractional step.

Each function returns a case description (faces, Reynolds number, time
step, boundary conditions, body, initial state, solver settings) that the
solver (IBMSolver via ``build_solver``) and the CPU oracle both consume.
The public benchmark configurations are seeded synthetic stand-ins: there is
no dataset to download.

* ``cavity``  - lid-driven cavity, uniform grid (the reference's
  src/cavity.c set-up: lid u=1 on the top face, walls elsewhere).
* ``sphere``  - flow past a sphere: domain [-5,15]x[-5,5]^2, cells
  clustered around the body, a 5-times subdivided icosphere (20480
  triangles, r = 0.5), uniform inflow on the west face, pressure outlet on
  the east face (the reference has no convective outflow; its sphere driver
  uses BC_PRESSURE, src/main.c:138-140), free-slip sides, Re 300.
* ``channel`` - channel LES: 2pi x 2 x pi, tanh-stretched walls in y,
  periodic x and z, constant body force 2/Re, Smagorinsky Cs = 0.1.
* ``ensemble`` - 64 independent immersed-body cases of uneven size (boxes
  or spheres, Re 50-500) for batched stepping.
"""
from __future__ import annotations

import os
import tempfile

import numpy as np

from . import geometry

_STL_CACHE = {}


def icosphere_stl(subdivisions=5, radius=0.5, center=(0.0, 0.0, 0.0)):
    key = (subdivisions, radius, tuple(center))
    path = _STL_CACHE.get(key)
    if path is None or not os.path.exists(path):
        fd, path = tempfile.mkstemp(prefix="icosphere%d_" % subdivisions, suffix=".stl")
        os.close(fd)
        geometry.write_stl(path, *geometry.icosphere(subdivisions, radius, center))
        _STL_CACHE[key] = path
    return path


def bumpy_stl(subdivisions=6, radius=0.5):
    """A large dented body (geometry.bumpy_sphere): 81,920 triangles for 6
    subdivisions, 327,680 for 7."""
    key = ("bumpy", subdivisions, radius)
    path = _STL_CACHE.get(key)
    if path is None or not os.path.exists(path):
        fd, path = tempfile.mkstemp(prefix="bumpy%d_" % subdivisions, suffix=".stl")
        os.close(fd)
        geometry.write_stl(path, *geometry.bumpy_sphere(subdivisions, radius))
        _STL_CACHE[key] = path
    return path


def cavity(n=64, Re=1000.0, dt=1e-3):
    f = geometry.uniform_faces(0.0, 1.0, n)
    return dict(name=f"cavity{n}", xf=f, yf=f.copy(), zf=f.copy(), re=Re, dt=dt,
                bc=["W wall", "E wall", "S wall", "N wall", "D wall", "U vel 1 0 0"],
                init=(0.0, 0.0, 0.0, 0.0))


def sphere(nx=192, ny=128, nz=128, Re=300.0, dt=5e-3, subdivisions=5):
    return dict(name=f"sphere{nx}x{ny}x{nz}",
                xf=geometry.body_clustered_faces(-5.0, 15.0, nx, 0.0, 3.0, 4.0),
                yf=geometry.body_clustered_faces(-5.0, 5.0, ny, 0.0, 3.0, 4.0),
                zf=geometry.body_clustered_faces(-5.0, 5.0, nz, 0.0, 3.0, 4.0),
                re=Re, dt=dt,
                bc=["W vel 1 0 0", "E press 0", "S slip", "N slip", "D slip", "U slip"],
                stl=icosphere_stl(subdivisions, 0.5), init=(1.0, 0.0, 0.0, 0.0))


def channel(nx=128, ny=96, nz=128, Re=16200.0, dt=2e-3, cs=0.1):
    return dict(name=f"channel{nx}x{ny}x{nz}",
                xf=geometry.uniform_faces(0.0, 2 * np.pi, nx), yf=geometry.tanh_faces(ny, 2.0),
                zf=geometry.uniform_faces(0.0, np.pi, nz), re=Re, dt=dt, force=(2.0 / Re, 0.0, 0.0),
                smag=cs, bc=["W per", "E per", "S wall", "N wall", "D per", "U per"],
                init="poiseuille")


def _body_stl(kind, params, key):
    """STL file of a synthetic body (cached per key)."""
    path = _STL_CACHE.get(key)
    if path is None or not os.path.exists(path):
        fd, path = tempfile.mkstemp(prefix=f"{kind}_", suffix=".stl")
        os.close(fd)
        if kind == "sphere":
            v, f = geometry.icosphere(params["subdivisions"], params["radius"], params["center"])
        else:
            v, f = geometry.box_union(params["boxes"])
        geometry.write_stl(path, v, f)
        _STL_CACHE[key] = path
    return path


def _boxes(rng, nbox, lo=-1.8, hi=1.8, gap=0.15, tries=200):
    """1-4 axis-aligned boxes with sides U[0.5, 2] inside [lo, hi]^3 that
    neither overlap nor touch (a gap of at least `gap`)."""
    out = []
    for _ in range(tries):
        if len(out) == nbox:
            break
        side = rng.uniform(0.5, 2.0, size=3)
        c = rng.uniform(lo + side / 2, hi - side / 2)
        b = (c - side / 2, c + side / 2)
        if all(np.any(b[0] > o[1] + gap) or np.any(o[0] > b[1] + gap) for o in out):
            out.append(b)
    return [(tuple(map(float, b[0])), tuple(map(float, b[1]))) for b in out]


def ensemble(ncases=64, seed=2024):
    """Seeded ensemble of independent immersed-body cases: grids
    Nx ~ U[32, 96], Ny, Nz ~ U[32, 64] on [-4, 8] x [-3, 3]^2, Re ~ U[50, 500],
    body = 1-4 non-touching boxes of side U[0.5, 2] or a sphere of diameter
    U[0.5, 1.5] (3-times subdivided icosphere), uniform inflow, pressure
    outlet, free-slip sides, dt = CFL 0.25 on the finest spacing."""
    rng = np.random.Generator(np.random.Philox(seed))
    cases = []
    for c in range(ncases):
        nx = int(rng.integers(32, 97))
        ny = int(rng.integers(32, 65))
        nz = int(rng.integers(32, 65))
        Re = float(rng.uniform(50.0, 500.0))
        xf = geometry.uniform_faces(-4.0, 8.0, nx)
        yf = geometry.uniform_faces(-3.0, 3.0, ny)
        zf = geometry.uniform_faces(-3.0, 3.0, nz)
        h = min(12.0 / nx, 6.0 / ny, 6.0 / nz)
        if rng.uniform() < 0.5:
            d = float(rng.uniform(0.5, 1.5))
            stl = _body_stl("sphere", dict(subdivisions=3, radius=d / 2, center=(0.0, 0.0, 0.0)),
                            ("sphere", round(d, 12)))
            body = f"sphere D={d:.3f}"
        else:
            boxes = _boxes(rng, int(rng.integers(1, 5)))
            stl = _body_stl("boxes", dict(boxes=boxes), ("boxes", tuple(boxes)))
            body = f"{len(boxes)} boxes"
        cases.append(dict(name=f"ens{c:02d}_{nx}x{ny}x{nz}", xf=xf, yf=yf, zf=zf, re=Re, dt=0.25 * h,
                          bc=["W vel 1 0 0", "E press 0", "S slip", "N slip", "D slip", "U slip"],
                          stl=stl, init=(1.0, 0.0, 0.0, 0.0), body=body))
    return cases


_BC = {"vel": "BC_VELOCITY_COMPONENT", "press": "BC_PRESSURE", "wall": "BC_STATIONARY_WALL",
       "slip": "BC_FREE_SLIP_WALL", "sym": "BC_SYMMETRIC", "per": "BC_ALL_PERIODIC",
       "velper": "BC_VELOCITY_PERIODIC"}
_DIR = {"N": "DIR_NORTH", "E": "DIR_EAST", "S": "DIR_SOUTH", "W": "DIR_WEST", "D": "DIR_DOWN", "U": "DIR_UP"}


def build_solver(ibm, case, tol=1e-6, div_tol=0.0, coarsening=None):
    """Create and assemble an IBMSolver for ``case`` (ibm = the package);
    coarsening: the pressure multigrid's mode, or (mode, width_ratio)
    (library default when None)."""
    s = ibm.IBMSolver()
    s.set_grid(case["xf"], case["yf"], case["zf"])
    s.set_params(case["re"], case["dt"])
    s.set_ext_force(*case.get("force", (0.0, 0.0, 0.0)))
    if "smag" in case:
        s.set_turb_model(ibm.TURBMODEL_SMAGORINSKY, case["smag"])
    for b in case["bc"]:
        t = b.split()
        s.set_bc(getattr(ibm, _DIR[t[0]]), getattr(ibm, _BC[t[1]]), *[float(v) for v in t[2:]])
    if case.get("stl"):
        s.set_obstacle(ibm.Polyhedron(case["stl"]))
    s.set_linear_solver(ibm.SOLVER_BiCGSTAB, ibm.PRECOND_AMG, tol)
    if div_tol > 0:
        s.set_div_tol(div_tol)
    if isinstance(coarsening, tuple):            # (mode, width_ratio)
        s.set_coarsening(*coarsening)
    elif coarsening is not None:
        s.set_coarsening(coarsening)
    s.assemble()
    return s


def initial_state(case, seed=0):
    """Initial (u1, u2, u3, p) in the padded layout."""
    nx, ny, nz = len(case["xf"]) - 1, len(case["yf"]) - 1, len(case["zf"]) - 1
    shape = (nx + 4, ny + 4, nz + 4)
    init = case.get("init", (0.0, 0.0, 0.0, 0.0))
    if init == "poiseuille":
        # Laminar profile 1 - y^2 plus 10% uniform noise from a seeded
        # counter-based generator (identical on every host).
        yf = np.asarray(case["yf"])
        yc = np.empty(ny + 4)
        yc[2:-2] = (yf[1:] + yf[:-1]) / 2
        yc[:2], yc[-2:] = yc[2], yc[-3]
        rng = np.random.Generator(np.random.Philox(seed))
        u = np.broadcast_to((1 - yc ** 2)[None, :, None], shape).copy()
        noise = rng.uniform(-0.1, 0.1, size=(3,) + shape)
        return u + noise[0], noise[1], noise[2], np.zeros(shape)
    return tuple(np.full(shape, float(v)) for v in init)
