"""The C-ABI library builds, loads without a GPU, and exports every entry
point that include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re

from conftest import ROOT, package


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:IBMSolver|Polyhedron|Vector)_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_reference_api():
    names = declared_functions()
    # The reference's public entry points (src/ibm3d_setup.h, ibm3d_init.h,
    # ibm3d_fracstep.h, ibm3d_turb.h, ibm3d_export.h, geo3d.h).
    ref = {"IBMSolver_new", "IBMSolver_destroy", "IBMSolver_set_grid", "IBMSolver_set_params",
           "IBMSolver_set_ext_force", "IBMSolver_set_turb_model", "IBMSolver_set_bc", "IBMSolver_set_obstacle",
           "IBMSolver_set_linear_solver", "IBMSolver_set_autosave", "IBMSolver_assemble",
           "IBMSolver_ghost_interp", "IBMSolver_init_flow_const", "IBMSolver_init_flow_file",
           "IBMSolver_init_flow_func", "IBMSolver_iterate", "IBMSolver_calc_tau_r",
           "IBMSolver_export_result", "IBMSolver_export_lvset_flag", "IBMSolver_export_intermediate",
           "Polyhedron_new", "Polyhedron_destroy", "Polyhedron_read_stl", "Polyhedron_print_stats",
           "Polyhedron_scale", "Polyhedron_cpt", "Vector_add", "Vector_sub", "Vector_dot", "Vector_crs",
           "Vector_norm", "Vector_dist", "Vector_angle", "Vector_normalize", "Vector_lincom", "Vector_rot"}
    assert ref <= names, sorted(ref - names)


def test_library_exports_every_declared_symbol():
    ibm = package()
    if not os.path.exists(ibm.LIB_PATH):
        importlib_build = __import__("importlib").import_module("2020researchproject_gb300.build")
        importlib_build.build()
    lib = ctypes.CDLL(ibm.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_enum_values_match_reference():
    ibm = package()
    assert (ibm.DIR_NORTH, ibm.DIR_EAST, ibm.DIR_SOUTH, ibm.DIR_WEST, ibm.DIR_DOWN, ibm.DIR_UP) == (1, 2, 4, 8, 16, 32)
    assert ibm.BC_VELOCITY_PERIODIC == 6 and ibm.BC_ALL_PERIODIC == 5 and ibm.BC_PRESSURE == 1
    assert (ibm.FLAG_FLUID, ibm.FLAG_GHOST, ibm.FLAG_SOLID) == (1, 2, 3)
    assert ibm.SOLVER_BiCGSTAB == 2 and ibm.PRECOND_AMG == 1
