"""Builds the C case driver (tests/drivers/ibm3d_driver.c) against the
public headers in include/ and the in-tree library, as a C host would."""
import os
import subprocess

from conftest import ROOT, package

DRIVER_SRC = os.path.join(ROOT, "tests", "drivers", "ibm3d_driver.c")


def library_path():
    ibm = package()
    if not os.path.exists(ibm.LIB_PATH):
        __import__("importlib").import_module("2020researchproject_gb300.build").build()
    return ibm.LIB_PATH


def compile_c(src, exe, extra=()):
    """gcc -std=gnu11 against include/ and libibm3d_gb300.so; returns the
    completed process (stdout/stderr captured)."""
    lib = library_path()
    cmd = ["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror=implicit-function-declaration",
           "-Werror=incompatible-pointer-types", *extra, "-I" + os.path.join(ROOT, "include"), "-o", exe, src, lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-lm"]
    return subprocess.run(cmd, capture_output=True, text=True)


def build_driver(tmpdir):
    exe = os.path.join(str(tmpdir), "ibm3d_driver")
    r = compile_c(DRIVER_SRC, exe, extra=("-Werror",))
    assert r.returncode == 0, r.stderr
    return exe
