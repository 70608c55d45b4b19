"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.  The oracle is a
plain-C restatement of the reference's time step (ibm3d_oracle.c) whose
parity is pinned to the golden fixtures produced by the reference itself.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

BC_TYPES = {"vel": 0, "press": 1, "wall": 2, "slip": 3, "sym": 4, "per": 5, "velper": 6}
FACES = {"N": 0, "E": 1, "S": 2, "W": 3, "D": 4, "U": 5}


class _Cfg(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("xf", ctypes.c_void_p), ("yf", ctypes.c_void_p), ("zf", ctypes.c_void_p),
                ("Re", ctypes.c_double), ("dt", ctypes.c_double),
                ("bc_type", ctypes.c_int * 6), ("bc_u", (ctypes.c_double * 3) * 6), ("bc_p", ctypes.c_double * 6),
                ("force", ctypes.c_double * 3), ("smagorinsky_cs", ctypes.c_double),
                ("tol", ctypes.c_double), ("div_tol", ctypes.c_double),
                ("stl_path", ctypes.c_char_p), ("lvset_in", ctypes.c_void_p), ("threads", ctypes.c_int),
                ("bc_fn", (ctypes.c_void_p * 4) * 6), ("force_fn", ctypes.c_void_p * 3)]

# double f(double t, double x, double y, double z)
_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double)


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "ibm3d_oracle.c")):
            subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
        lib = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        lib.oracle_create.restype = vp
        lib.oracle_create.argtypes = [ctypes.POINTER(_Cfg)]
        lib.oracle_destroy.argtypes = [vp]
        lib.oracle_init.argtypes = [vp, vp, vp, vp, vp]
        lib.oracle_iterate.argtypes = [vp, ctypes.c_int]
        lib.oracle_get.restype = ctypes.c_int
        lib.oracle_get.argtypes = [vp, ctypes.c_char_p, vp]
        lib.oracle_flag.argtypes = [vp, vp]
        lib.oracle_num_ghost.restype = ctypes.c_int
        lib.oracle_num_ghost.argtypes = [vp]
        lib.oracle_ghost_stencils.argtypes = [vp, vp, vp, vp]
        lib.oracle_stats.argtypes = [vp, vp, vp, vp]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """case: dict with grid faces xf/yf/zf, re, dt, bc (list like "W vel 1 0 0"),
    optional force, smag, stl (path), tol, div_tol, lvset (padded array), threads,
    bc_funcs (list of (face, type, callables): VAL_FUNC faces, three callables
    f(t, x, y, z) for "vel", one for "press" / "velper") and force_funcs
    (three callables)."""

    def __init__(self, case):
        lib = load()
        self._keep = []
        c = _Cfg()
        xf, yf, zf = (np.ascontiguousarray(case[k], dtype=np.float64) for k in ("xf", "yf", "zf"))
        self._keep += [xf, yf, zf]
        c.nx, c.ny, c.nz = len(xf) - 1, len(yf) - 1, len(zf) - 1
        self.shape = (c.nx, c.ny, c.nz)
        c.xf, c.yf, c.zf = _p(xf), _p(yf), _p(zf)
        c.Re, c.dt = float(case["re"]), float(case["dt"])
        for b in case["bc"]:
            t = b.split()
            f = FACES[t[0]]
            c.bc_type[f] = BC_TYPES[t[1]]
            vals = [float(v) for v in t[2:]]
            if t[1] == "vel":
                for l in range(3):
                    c.bc_u[f][l] = vals[l]
            elif t[1] in ("press", "velper"):
                c.bc_p[f] = vals[0]
        for face, kind, fns in case.get("bc_funcs", []):
            f = FACES[face]
            c.bc_type[f] = BC_TYPES[kind]
            slots = range(3) if kind == "vel" else (3,)
            for q, fn in zip(slots, fns):
                cb = _FN(fn)
                self._keep.append(cb)
                c.bc_fn[f][q] = ctypes.cast(cb, ctypes.c_void_p)
        for l, v in enumerate(case.get("force", (0, 0, 0))):
            c.force[l] = float(v)
        for l, fn in enumerate(case.get("force_funcs", ())):
            cb = _FN(fn)
            self._keep.append(cb)
            c.force_fn[l] = ctypes.cast(cb, ctypes.c_void_p)
        c.smagorinsky_cs = float(case.get("smag", -1.0))
        c.tol = float(case.get("tol", 1e-12))
        c.div_tol = float(case.get("div_tol", 0.0))
        stl = case.get("stl")
        c.stl_path = stl.encode() if stl else None
        lv = case.get("lvset")
        if lv is not None:
            lv = np.ascontiguousarray(lv, dtype=np.float64)
            self._keep.append(lv)
            c.lvset_in = _p(lv)
        c.threads = int(case.get("threads", 0))
        self._o = lib.oracle_create(ctypes.byref(c))

    def __del__(self):
        if getattr(self, "_o", None):
            load().oracle_destroy(self._o)
            self._o = None

    def init(self, u1, u2, u3, p):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u1, u2, u3, p)]
        load().oracle_init(self._o, *(_p(a) for a in arrs))

    def iterate(self, n):
        load().oracle_iterate(self._o, int(n))

    def get(self, name):
        nx, ny, nz = self.shape
        shape = {"U1": (nx + 1, ny + 4, nz + 4), "U2": (nx + 4, ny + 1, nz + 4),
                 "U3": (nx + 4, ny + 4, nz + 1)}.get(name[:2] if name[0] == "U" else "", (nx + 4, ny + 4, nz + 4))
        out = np.empty(shape, dtype=np.float64)
        if load().oracle_get(self._o, name.encode(), _p(out)) != 0:
            raise KeyError(name)
        return out

    def flag(self):
        nx, ny, nz = self.shape
        out = np.empty((nx + 4, ny + 4, nz + 4), dtype=np.int32)
        load().oracle_flag(self._o, _p(out))
        return out

    def ghost_stencils(self):
        n = load().oracle_num_ghost(self._o)
        ijk = np.empty((n, 3), dtype=np.int32)
        idx = np.empty((n, 8, 3), dtype=np.int32)
        coeff = np.empty((n, 8), dtype=np.float64)
        if n:
            load().oracle_ghost_stencils(self._o, _p(ijk), _p(idx), _p(coeff))
        return ijk, idx, coeff

    def stats(self):
        it = np.zeros(4, dtype=np.int32)
        res = np.zeros(4, dtype=np.float64)
        md = ctypes.c_double()
        load().oracle_stats(self._o, _p(it), _p(res), ctypes.byref(md))
        return dict(iters=it.tolist(), res=res.tolist(), max_div=md.value)
