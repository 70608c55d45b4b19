"""ibm3d-gb300: the reference's 3D immersed-boundary fractional step on one GB300.

Python mirror of the C ABI in include/ibm3d.h (the reference's
``IBMSolver_*`` / ``Polyhedron_*`` API) over ctypes.  The compute path is
the in-tree CUDA library ``libibm3d_gb300.so``; there is no CPU fallback:
importing works anywhere, but creating a solver without the library or
without a GPU raises.

    import importlib
    ibm = importlib.import_module("2020researchproject_gb300")
    s = ibm.IBMSolver()
    s.set_grid(xf, yf, zf); s.set_params(Re, dt)
    s.set_bc(ibm.DIR_UP, ibm.BC_VELOCITY_COMPONENT, 1, 0, 0)
    ...
    s.assemble(); s.init_flow_const(0, 0, 0, 0); s.iterate(10)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

# Batched steps run one graph branch (or stream) per member: let the GPU
# work on up to 32 of them at once (CUDA's default is 8 hardware queues).
# Set on import, before anything in this process creates a CUDA context.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libibm3d_gb300.so")

# Enums, values as in the reference's src/ibm3d.h:16-98.
SOLVER_AMG, SOLVER_PCG, SOLVER_BiCGSTAB, SOLVER_GMRES = range(4)
PRECOND_NONE, PRECOND_AMG = range(2)
FP64, MIXED, MIXED_MG, MIXED32, MIXED32_IR = 0, 1, 2, 3, 4
PVEC_FP64, PVEC_DFLOAT = 0, 1
COARSEN_HALVE, COARSEN_SPACING = 0, 1
DIR_NORTH, DIR_EAST, DIR_SOUTH, DIR_WEST, DIR_DOWN, DIR_UP = (1 << i for i in range(6))
(BC_VELOCITY_COMPONENT, BC_PRESSURE, BC_STATIONARY_WALL, BC_FREE_SLIP_WALL,
 BC_SYMMETRIC, BC_ALL_PERIODIC, BC_VELOCITY_PERIODIC) = range(7)
VAL_CONST, VAL_FUNC = range(2)
TURBMODEL_NONE, TURBMODEL_SMAGORINSKY, TURBMODEL_WALE = range(3)
FLAG_FLUID, FLAG_GHOST, FLAG_SOLID = 1, 2, 3

# Extension enums (include/ibm3d_gb300.h).
FIELDS = ["u1", "u2", "u3", "p", "U1", "U2", "U3", "u1star", "u2star", "u3star",
          "U1star", "U2star", "U3star", "pprime", "N1", "N2", "N3", "lvset", "coeffsum",
          "tau11", "tau12", "tau13", "tau22", "tau23", "tau33"]
STATUS = {0: "ok", 1: "no convergence", 2: "breakdown", 3: "CUDA error", 4: "invalid argument",
          5: "mirror point outside grid", 6: "unsupported", 7: "non-finite values"}


class IBM3DError(RuntimeError):
    pass


# double f(double t, double x, double y, double z): IBMSolverBCValFunc and
# IBMSolverForceFunc (src/ibm3d.h).
_VALFUNC = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double)


class _Stats(ctypes.Structure):
    _fields_ = [("iter", ctypes.c_int), ("time", ctypes.c_double),
                ("iters_u", ctypes.c_int * 3), ("iters_p", ctypes.c_int),
                ("res_u", ctypes.c_double * 3), ("res_p", ctypes.c_double),
                ("max_div", ctypes.c_double), ("mg_levels", ctypes.c_int),
                ("cpt_fallback", ctypes.c_int), ("outer_u", ctypes.c_int),
                ("outer_p", ctypes.c_int), ("steps_total", ctypes.c_longlong),
                ("iters_u_total", ctypes.c_longlong * 3), ("iters_p_total", ctypes.c_longlong),
                ("outer_p_total", ctypes.c_longlong), ("max_div_max", ctypes.c_double)]


_lib = None


def library_loaded() -> bool:
    return _lib is not None


def load_library(path: str = LIB_PATH):
    """Load (once) the CUDA library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise IBM3DError(f"{path} is missing: run __graft_entry__.build() "
                         "(the GB300 path has no CPU fallback)")
    os.environ.setdefault("IBM3D_NO_ABORT", "1")
    lib = ctypes.CDLL(path)
    vp, d, i, dp, ip = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p
    sig = {
        "IBMSolver_new": (vp, [i, i, i, i, i]),
        "IBMSolver_destroy": (None, [vp]),
        "IBMSolver_set_grid": (None, [vp, i, i, i, dp, dp, dp]),
        "IBMSolver_set_params": (None, [vp, d, d]),
        "IBMSolver_set_bc_const": (None, [vp, i, i, d, d, d, d]),
        "IBMSolver_set_ext_force_const": (None, [vp, d, d, d]),
        "IBMSolver_set_bc_func": (None, [vp, i, i, vp, vp, vp, vp]),
        "IBMSolver_set_refinement": (None, [vp, d, d, i]),
        "IBMSolver_set_gmres_restart": (None, [vp, i]),
        "IBMSolver_set_coarsening": (None, [vp, i, d]),
        "IBMSolver_set_warm_start": (None, [vp, i]),
        "IBMSolver_set_max_iters": (None, [vp, i, i]),
        "IBMSolver_set_pressure_guess": (None, [vp, i]),
        "IBMSolver_set_pressure_vectors": (None, [vp, i]),
        "IBMSolver_measure_fma_rate": (d, [i]),
        "IBMSolver_check_fp32_conversions": (i, [ctypes.c_longlong, dp, ctypes.POINTER(ctypes.c_ulonglong)]),
        "IBMSolver_autotune": (d, [vp, i, ip]),
        "IBMSolver_set_ext_force_func": (None, [vp, vp, vp, vp]),
        "IBMSolver_set_smagorinsky": (None, [vp, d]),
        "IBMSolver_set_obstacle": (None, [vp, vp]),
        "IBMSolver_set_linear_solver": (None, [vp, i, i, d]),
        "IBMSolver_set_autosave": (None, [vp, ctypes.c_char_p, i]),
        "IBMSolver_assemble": (None, [vp]),
        "IBMSolver_ghost_interp": (None, [vp, i, i, i, ip, dp]),
        "IBMSolver_init_flow_const": (None, [vp, d, d, d, d]),
        "IBMSolver_init_flow_array": (None, [vp, dp, dp, dp, dp]),
        "IBMSolver_init_flow_file": (None, [vp, ctypes.c_char_p]),
        "IBMSolver_iterate": (None, [vp, i, ctypes.c_bool]),
        "IBMSolver_calc_tau_r": (None, [vp]),
        "IBMSolver_export_result": (None, [vp, ctypes.c_char_p]),
        "IBMSolver_export_lvset_flag": (None, [vp, ctypes.c_char_p]),
        "IBMSolver_export_intermediate": (None, [vp, ctypes.c_char_p]),
        "IBMSolver_last_status": (i, [vp]),
        "IBMSolver_last_message": (ctypes.c_char_p, [vp]),
        "IBMSolver_set_div_tol": (None, [vp, d]),
        "IBMSolver_set_precision": (None, [vp, i]),
        "IBMSolver_set_graphs": (None, [vp, i]),
        "IBMSolver_time_kernel": (ctypes.c_double, [vp, i, i, ctypes.POINTER(ctypes.c_double)]),
        "IBMSolver_set_multigrid": (None, [vp, i, i, i, i, i, ctypes.c_double]),
        "IBMSolver_get_field": (None, [vp, i, dp]),
        "IBMSolver_get_flag": (None, [vp, ip]),
        "IBMSolver_sync_host": (None, [vp]),
        "IBMSolver_num_ghost": (i, [vp]),
        "IBMSolver_num_ghost_levels": (i, [vp]),
        "IBMSolver_get_ghost_stencils": (None, [vp, ip, ip, dp]),
        "IBMSolver_get_stats": (None, [vp, ctypes.POINTER(_Stats)]),
        "IBMSolver_time_iterate": (d, [vp, i]),
        "IBMSolver_set_profiling": (None, [vp, i]),
        "IBMSolver_get_profile": (i, [vp, i, vp, ip, dp]),
        "IBMSolver_device_name": (ctypes.c_char_p, [vp]),
        "IBMSolver_kernel_launches": (ctypes.c_longlong, []),
        "IBMSolver_host_register": (i, [vp, ctypes.c_size_t]),
        "IBMSolver_host_unregister": (i, [vp]),
        "IBMSolver_device_bytes": (ctypes.c_size_t, [vp]),
        "IBMBatch_new": (vp, []),
        "IBMBatch_destroy": (None, [vp]),
        "IBMBatch_add": (i, [vp, vp]),
        "IBMBatch_remove": (i, [vp, vp]),
        "IBMBatch_size": (i, [vp]),
        "IBMBatch_iterate": (d, [vp, i]),
        "IBMBatch_launch": (i, [vp]),
        "IBMBatch_wait": (i, [vp]),
        "IBMBatch_last_status": (i, [vp]),
        "IBMBatch_set_combined": (None, [vp, i]),
        "Polyhedron_new": (vp, []),
        "Polyhedron_destroy": (None, [vp]),
        "Polyhedron_read_stl": (None, [vp, vp]),
        "Polyhedron_cpt": (None, [vp, i, i, i, dp, dp, dp, dp, d]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def kernel_launches() -> int:
    """Kernels the library has launched since it was loaded."""
    return int(load_library().IBMSolver_kernel_launches())


def measure_fma_rate(fp64=True) -> float:
    """Register-only FMA throughput of the GPU in TFLOP/s (FP64 or FP32)."""
    return float(load_library().IBMSolver_measure_fma_rate(0 if fp64 else 1))


def check_fp32_conversions(values) -> int:
    """Mismatches between the integer-pipe FP64 <-> FP32 conversions of the
    IBM3D_MIXED32 step and the GPU's conversion instructions on `values`."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    bad = ctypes.c_ulonglong(0)
    if load_library().IBMSolver_check_fp32_conversions(len(v), _ptr(v), ctypes.byref(bad)) != 0:
        raise IBM3DError("IBMSolver_check_fp32_conversions failed")
    return int(bad.value)


def pin(a: np.ndarray) -> bool:
    """Page-lock a numpy array's memory for direct host<->device DMA."""
    return load_library().IBMSolver_host_register(a.ctypes.data_as(ctypes.c_void_p), a.nbytes) == 0


def unpin(a: np.ndarray) -> None:
    load_library().IBMSolver_host_unregister(a.ctypes.data_as(ctypes.c_void_p))


class Polyhedron:
    """Binary-STL body (src/geo3d.h Polyhedron API)."""

    def __init__(self, path: str):
        lib = load_library()
        libc = ctypes.CDLL(None)
        libc.fopen.restype = ctypes.c_void_p
        libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        libc.fclose.argtypes = [ctypes.c_void_p]
        fp = libc.fopen(path.encode(), b"rb")
        if not fp:
            raise IBM3DError(f"cannot open {path}")
        self._p = lib.Polyhedron_new()
        lib.Polyhedron_read_stl(self._p, fp)
        libc.fclose(fp)

    def cpt(self, x, y, z, maxd=15.0):
        """Signed distance on the grid x[i], y[j], z[k] (GPU)."""
        lib = load_library()
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        f = np.empty((len(x), len(y), len(z)), dtype=np.float64)
        lib.Polyhedron_cpt(self._p, len(x), len(y), len(z), _ptr(x), _ptr(y), _ptr(z), _ptr(f), maxd)
        return f

    def __del__(self):
        if getattr(self, "_p", None) and _lib is not None:
            _lib.Polyhedron_destroy(self._p)
            self._p = None


class IBMSolver:
    """One solver instance; method names follow IBMSolver_<name> of the C ABI."""

    def __init__(self, num_process=1, rank=0, Px=1, Py=1, Pz=1):
        self._lib = load_library()
        self._s = self._lib.IBMSolver_new(num_process, rank, Px, Py, Pz)
        self._check("IBMSolver_new")
        self.shape = None
        self._callbacks = []

    def _check(self, what):
        st = self._lib.IBMSolver_last_status(self._s)
        if st not in (0, 1):
            msg = self._lib.IBMSolver_last_message(self._s) or b""
            raise IBM3DError(f"{what}: {STATUS.get(st, st)}: {msg.decode(errors='replace')}")

    def close(self):
        """Destroys the solver now (frees its device memory)."""
        if getattr(self, "_s", None):
            self._lib.IBMSolver_destroy(self._s)
            self._s = None

    def __del__(self):
        self.close()

    # ------------------------------------------------------------ setup
    def set_grid(self, xf, yf, zf):
        self._xf, self._yf, self._zf = (np.ascontiguousarray(a, dtype=np.float64) for a in (xf, yf, zf))
        nx, ny, nz = len(self._xf) - 1, len(self._yf) - 1, len(self._zf) - 1
        self.shape = (nx, ny, nz)
        self._lib.IBMSolver_set_grid(self._s, nx, ny, nz, _ptr(self._xf), _ptr(self._yf), _ptr(self._zf))
        self._check("set_grid")

    def set_params(self, Re, dt):
        self._lib.IBMSolver_set_params(self._s, Re, dt)

    def _func(self, f):
        """A C callback double(t, x, y, z) for f, kept alive with the solver."""
        cb = _VALFUNC(f)
        self._callbacks.append(cb)
        return ctypes.cast(cb, ctypes.c_void_p)

    def set_bc(self, direction, bc_type, *values):
        """set_bc(DIR, BC_VELOCITY_COMPONENT, u1, u2, u3) | (DIR, BC_PRESSURE, p)
        | (DIR, BC_VELOCITY_PERIODIC, p) | (DIR, other type).  Values are
        numbers (VAL_CONST) or callables f(t, x, y, z) (VAL_FUNC)."""
        if values and all(callable(v) for v in values):
            fs = [self._func(v) for v in values]
            if bc_type == BC_VELOCITY_COMPONENT:
                self._lib.IBMSolver_set_bc_func(self._s, direction, bc_type, fs[0], fs[1], fs[2], None)
            else:
                self._lib.IBMSolver_set_bc_func(self._s, direction, bc_type, None, None, None, fs[0])
            self._check("set_bc")
            return
        u = [0.0, 0.0, 0.0]
        p = 0.0
        if bc_type == BC_VELOCITY_COMPONENT:
            u = [float(v) for v in values]
        elif bc_type in (BC_PRESSURE, BC_VELOCITY_PERIODIC):
            p = float(values[0])
        self._lib.IBMSolver_set_bc_const(self._s, direction, bc_type, u[0], u[1], u[2], p)

    def set_ext_force(self, f1, f2, f3):
        """Constant force components, or callables f(t, x, y, z) (VAL_FUNC)."""
        if all(callable(f) for f in (f1, f2, f3)):
            self._lib.IBMSolver_set_ext_force_func(self._s, *(self._func(f) for f in (f1, f2, f3)))
        else:
            self._lib.IBMSolver_set_ext_force_const(self._s, f1, f2, f3)

    def set_turb_model(self, model, Cs=0.0):
        if model == TURBMODEL_SMAGORINSKY:
            self._lib.IBMSolver_set_smagorinsky(self._s, Cs)
        elif model != TURBMODEL_NONE:
            raise IBM3DError("only TURBMODEL_NONE and TURBMODEL_SMAGORINSKY exist")

    def set_obstacle(self, poly):
        self._poly = poly
        self._lib.IBMSolver_set_obstacle(self._s, poly._p if poly is not None else None)

    def set_linear_solver(self, solver_type, precond_type, tol):
        self._lib.IBMSolver_set_linear_solver(self._s, solver_type, precond_type, tol)
        self._check("set_linear_solver")

    def set_div_tol(self, div_tol):
        self._lib.IBMSolver_set_div_tol(self._s, div_tol)

    def set_multigrid(self, nu_pre=3, nu_post=3, nuc_pre=2, nuc_post=2, coarse_sweeps=16, omega=1.0):
        self._lib.IBMSolver_set_multigrid(self._s, nu_pre, nu_post, nuc_pre, nuc_post, coarse_sweeps, float(omega))
        self._check("IBMSolver_set_multigrid")

    def time_kernel(self, which, reps=20, cold=False):
        """(avg ms per launch, algorithmic bytes per launch) of a hot kernel:
        which = "mg_color", "spmv_p", "conv_rhs", "ustar_prhs" or
        "update_next"; cold: the L2 is overwritten before each launch."""
        b = ctypes.c_double(0.0)
        code = {"mg_color": 0, "spmv_p": 1, "conv_rhs": 2, "ustar_prhs": 3, "update_next": 4}[which]
        if cold:
            code |= 256
        ms = self._lib.IBMSolver_time_kernel(self._s, code, int(reps), ctypes.byref(b))
        self._check("IBMSolver_time_kernel")
        return ms, b.value

    def autotune(self, steps=2):
        """Picks the multigrid sweeps by timing `steps` steps per candidate
        (state restored afterwards); returns (ms per step, sweeps)."""
        best = np.zeros(5, dtype=np.int32)
        ms = self._lib.IBMSolver_autotune(self._s, int(steps), _ptr(best))
        self._check("autotune")
        return ms, tuple(int(v) for v in best)

    def set_warm_start(self, on=True):
        """Mixed modes: momentum solve from the current velocity (default on)."""
        self._lib.IBMSolver_set_warm_start(self._s, 1 if on else 0)
        self._check("set_warm_start")

    def set_pressure_guess(self, mode=1):
        """Warm-started pressure solves from the last increment (0) or its
        linear extrapolation from the last two (1, the default)."""
        self._lib.IBMSolver_set_pressure_guess(self._s, int(mode))
        self._check("set_pressure_guess")

    def set_pressure_vectors(self, kind=PVEC_DFLOAT):
        """MIXED32 pressure BiCGSTAB vectors: double-float (default) or FP64."""
        self._lib.IBMSolver_set_pressure_vectors(self._s, int(kind))
        self._check("set_pressure_vectors")

    def set_max_iters(self, max_mom=200, max_p=1000):
        """Krylov iteration caps (the reference's 200 and 1000 by default)."""
        self._lib.IBMSolver_set_max_iters(self._s, int(max_mom), int(max_p))
        self._check("set_max_iters")

    def set_coarsening(self, mode=COARSEN_SPACING, width_ratio=0.0):
        """Pressure multigrid coarsening (before assemble): COARSEN_SPACING
        (width_ratio: its merge threshold, 0 = default) or COARSEN_HALVE."""
        self._lib.IBMSolver_set_coarsening(self._s, int(mode), float(width_ratio))
        self._check("set_coarsening")

    def set_gmres_restart(self, restart=10):
        self._lib.IBMSolver_set_gmres_restart(self._s, restart)
        self._check("set_gmres_restart")

    def set_refinement(self, inner_tol_mom=5e-7, inner_tol_p=1e-5, max_outer=12):
        self._lib.IBMSolver_set_refinement(self._s, inner_tol_mom, inner_tol_p, max_outer)
        self._check("set_refinement")

    def set_graphs(self, on=True):
        self._lib.IBMSolver_set_graphs(self._s, 1 if on else 0)

    def set_precision(self, mode):
        self._lib.IBMSolver_set_precision(self._s, int(mode))
        self._check("IBMSolver_set_precision")

    def assemble(self):
        self._lib.IBMSolver_assemble(self._s)
        self._check("assemble")

    # ------------------------------------------------------------- init
    def init_flow_const(self, u1, u2, u3, p):
        self._lib.IBMSolver_init_flow_const(self._s, u1, u2, u3, p)
        self._check("init_flow_const")

    def init_flow_array(self, u1, u2, u3, p):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u1, u2, u3, p)]
        self._lib.IBMSolver_init_flow_array(self._s, *(_ptr(a) for a in arrs))
        self._check("init_flow_array")

    def init_flow_file(self, name):
        self._lib.IBMSolver_init_flow_file(self._s, name.encode())
        self._check("init_flow_file")

    # ------------------------------------------------------------- step
    def iterate(self, nsteps, verbose=False):
        self._lib.IBMSolver_iterate(self._s, nsteps, verbose)
        self._check("iterate")

    def time_iterate(self, nsteps):
        ms = self._lib.IBMSolver_time_iterate(self._s, nsteps)
        self._check("time_iterate")
        return ms

    def calc_tau_r(self):
        self._lib.IBMSolver_calc_tau_r(self._s)

    def export_result(self, name):
        self._lib.IBMSolver_export_result(self._s, name.encode())
        self._check("export_result")

    def export_lvset_flag(self, name):
        """"<name>.nc": level set and flags over the padded grid."""
        self._lib.IBMSolver_export_lvset_flag(self._s, name.encode())
        self._check("export_lvset_flag")

    def export_intermediate(self, name):
        """"<name>.nc": the last step's u*, u~ and p'."""
        self._lib.IBMSolver_export_intermediate(self._s, name.encode())
        self._check("export_intermediate")

    # ---------------------------------------------------------- readback
    def _field_shape(self, name):
        nx, ny, nz = self.shape
        return {"U1": (nx + 1, ny + 4, nz + 4), "U2": (nx + 4, ny + 1, nz + 4),
                "U3": (nx + 4, ny + 4, nz + 1)}.get(name[:2] if name[0] == "U" else "", (nx + 4, ny + 4, nz + 4))

    def get_field(self, name):
        out = np.empty(self._field_shape(name), dtype=np.float64)
        self._lib.IBMSolver_get_field(self._s, FIELDS.index(name), _ptr(out))
        self._check("get_field")
        return out

    def get_field_into(self, name, out):
        """Read a field into a caller-owned C-contiguous float64 array."""
        assert out.flags.c_contiguous and out.dtype == np.float64 and out.shape == self._field_shape(name)
        self._lib.IBMSolver_get_field(self._s, FIELDS.index(name), _ptr(out))
        self._check("get_field")
        return out

    def get_flag(self):
        nx, ny, nz = self.shape
        out = np.empty((nx + 4, ny + 4, nz + 4), dtype=np.int32)
        self._lib.IBMSolver_get_flag(self._s, _ptr(out))
        return out

    def ghost_stencils(self):
        n = self._lib.IBMSolver_num_ghost(self._s)
        ijk = np.empty((n, 3), dtype=np.int32)
        idx = np.empty((n, 8, 3), dtype=np.int32)
        coeff = np.empty((n, 8), dtype=np.float64)
        if n:
            self._lib.IBMSolver_get_ghost_stencils(self._s, _ptr(ijk), _ptr(idx), _ptr(coeff))
        return ijk, idx, coeff

    def num_ghost_levels(self):
        return self._lib.IBMSolver_num_ghost_levels(self._s)

    def ghost_interp(self, i, j, k):
        idx = np.empty((8, 3), dtype=np.int32)
        coeff = np.empty(8, dtype=np.float64)
        self._lib.IBMSolver_ghost_interp(self._s, i, j, k, _ptr(idx), _ptr(coeff))
        return idx, coeff

    def stats(self):
        st = _Stats()
        self._lib.IBMSolver_get_stats(self._s, ctypes.byref(st))
        return dict(iter=st.iter, time=st.time, iters_u=list(st.iters_u), iters_p=st.iters_p,
                    res_u=list(st.res_u), res_p=st.res_p, max_div=st.max_div,
                    mg_levels=st.mg_levels, cpt_fallback=st.cpt_fallback,
                    outer_u=st.outer_u, outer_p=st.outer_p, steps_total=st.steps_total,
                    iters_u_total=list(st.iters_u_total), iters_p_total=st.iters_p_total,
                    outer_p_total=st.outer_p_total, max_div_max=st.max_div_max)

    def device_bytes(self):
        """Device memory taken by assembly (bytes)."""
        return int(self._lib.IBMSolver_device_bytes(self._s))

    def set_profiling(self, on=True):
        self._lib.IBMSolver_set_profiling(self._s, 1 if on else 0)

    def profile(self):
        names = (ctypes.c_char * 32 * 64)()
        launches = np.zeros(64, dtype=np.int32)
        total = np.zeros(64, dtype=np.float64)
        n = self._lib.IBMSolver_get_profile(self._s, 64, names, _ptr(launches), _ptr(total))
        return {names[q].value.decode(): (int(launches[q]), float(total[q])) for q in range(n)}

    def device_name(self):
        return self._lib.IBMSolver_device_name(self._s).decode()


class Batch:
    """Independent solvers advanced together, one CUDA graph launch per
    batched step (IBMBatch_* of include/ibm3d_gb300.h).  Each member gets
    exactly the results IBMSolver.iterate gives it alone."""

    def __init__(self, solvers=(), combined=True):
        self._lib = load_library()
        self._b = self._lib.IBMBatch_new()
        self._members = []
        if not combined:
            self.set_combined(False)
        for s in solvers:
            self.add(s)

    def set_combined(self, on=True):
        """True: one graph launch per batched step (re-recorded on membership
        changes); False: each member's own step graph on its own stream."""
        self._lib.IBMBatch_set_combined(self._b, 1 if on else 0)

    def add(self, solver):
        if self._lib.IBMBatch_add(self._b, solver._s) != 0:
            raise IBM3DError("IBMBatch_add failed (solver not assembled?)")
        self._members.append(solver)

    def remove(self, solver):
        if self._lib.IBMBatch_remove(self._b, solver._s) != 0:
            raise IBM3DError("IBMBatch_remove: not a member")
        self._members.remove(solver)

    def __len__(self):
        return len(self._members)

    def iterate(self, nsteps=1):
        """Advances every member nsteps steps; returns device milliseconds."""
        ms = self._lib.IBMBatch_iterate(self._b, int(nsteps))
        st = self._lib.IBMBatch_last_status(self._b)
        if ms < 0 or st not in (0, 1):
            raise IBM3DError(f"IBMBatch_iterate: {STATUS.get(st, st)}")
        return ms

    def launch(self):
        """Queues one batched step and returns at once (see wait)."""
        if self._lib.IBMBatch_launch(self._b) != 0:
            raise IBM3DError("IBMBatch_launch failed")

    def wait(self):
        """Waits for the step queued by launch and books it."""
        rc = self._lib.IBMBatch_wait(self._b)
        st = self._lib.IBMBatch_last_status(self._b)
        if rc != 0 or st not in (0, 1):
            raise IBM3DError(f"IBMBatch_wait: {STATUS.get(st, st)}")

    def __del__(self):
        if getattr(self, "_b", None):
            self._lib.IBMBatch_destroy(self._b)
            self._b = None
