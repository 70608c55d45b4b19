"""The drop-in boundary from C: a driver written against include/ only
compiles and links with libibm3d_gb300.so, through the reference's
variadic set_bc / set_ext_force / set_turb_model conventions and the
MPI / hypre start-up calls of the reference's drivers; where the
reference's sources are available, its own five case drivers (src/main.c,
cavity.c, channel.c, jet.c, building.c) compile and link against this
library unchanged.  No GPU: nothing here runs a solver."""
import os
import shutil

import pytest

from c_driver import build_driver, compile_c

REF_SRC = os.environ.get("IBM3D_REF_SRC", "/root/reference/src")


def test_c_driver_builds(tmp_path):
    exe = build_driver(tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.parametrize("name", ["main", "cavity", "channel", "jet", "building"])
def test_reference_driver_compiles_unchanged(tmp_path, name):
    src = os.path.join(REF_SRC, name + ".c")
    if not os.path.exists(src):
        pytest.skip("the reference's sources are not mounted here")
    # A copy on its own, as in a user's project: its #include "ibm3d.h",
    # "utils.h", "geo3d.h" must resolve to this library's headers.
    local = os.path.join(str(tmp_path), name + ".c")
    shutil.copy(src, local)
    r = compile_c(local, os.path.join(str(tmp_path), name), extra=("-Wno-unused-result",))
    assert r.returncode == 0, r.stderr
