"""Build the in-tree GB300 library libibm3d_gb300.so (sm_103a only).

    python -m 2020researchproject_gb300.build      (or build() from Python)

Each translation unit compiles in parallel with nvcc/g++; objects go to
_build/ inside the package and the shared library next to this file.  The
set-up kernels are compiled with -fmad=false so that level sets, flags and
ghost stencils are computed without fused multiply-adds, like the
reference's C build.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libibm3d_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CUDA_SOURCES = {
    "step_kernels.cu": [],
    "step32_kernels.cu": [],
    "krylov.cu": [],
    "multigrid.cu": [],
    "setup_kernels.cu": ["-fmad=false"],
    "solver.cu": [],
}
CXX_SOURCES = ["geo3d.cpp", "ncfile.cpp", "utils_abi.cpp"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every translation unit for sm_103a and link the library.
    Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers += [os.path.join(PKG, "..", "include", h) for h in os.listdir(os.path.join(PKG, "..", "include"))]
    cmds, objs = [], []
    for src, extra in CUDA_SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmds.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "--extended-lambda",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", *extra, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-I/usr/local/cuda/include", "-I" + os.path.join(PKG, "..", "include"), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out.strip():
                print(out)
    if cmds or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
