"""Failure detection on the host, without a GPU: bad body files end the
process with the reference's fatal-error convention (a message on stderr
and a non-zero exit; the reference aborts its MPI job,
src/utils.c:13-20, src/geo3d.c:229-368), checked in child processes."""
import os
import subprocess
import sys

import numpy as np

from conftest import GOLDEN, ROOT

CHILD = """
import sys
sys.path.insert(0, {root!r})
import importlib
ibm = importlib.import_module("2020researchproject_gb300")
ibm.Polyhedron(sys.argv[1])
print("read ok")
"""


def _read_in_child(path):
    return subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT), path], capture_output=True, text=True,
                          timeout=120)


def _stl_records(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[80:84], np.uint32)[0])
    return b[:80], n, [b[84 + 50 * i:84 + 50 * (i + 1)] for i in range(n)]


def test_valid_stl_reads():
    r = _read_in_child(os.path.join(GOLDEN, "box.stl"))
    assert r.returncode == 0 and "read ok" in r.stdout, r.stderr


def test_truncated_stl_is_fatal(tmp_path):
    head, n, recs = _stl_records(os.path.join(GOLDEN, "box.stl"))
    bad = os.path.join(str(tmp_path), "truncated.stl")
    with open(bad, "wb") as fh:   # header promises n facets, the file holds n - 1 and a half
        fh.write(head + np.uint32(n).tobytes() + b"".join(recs[:-1]) + recs[-1][:20])
    r = _read_in_child(bad)
    assert r.returncode != 0 and "read ok" not in r.stdout
    assert "truncated STL" in r.stderr


def test_open_surface_is_fatal(tmp_path):
    head, n, recs = _stl_records(os.path.join(GOLDEN, "box.stl"))
    bad = os.path.join(str(tmp_path), "open.stl")
    with open(bad, "wb") as fh:   # one facet removed: the box is no longer closed
        fh.write(head + np.uint32(n - 1).tobytes() + b"".join(recs[:-1]))
    r = _read_in_child(bad)
    assert r.returncode != 0 and "read ok" not in r.stdout
    assert "not a closed 2-manifold" in r.stderr


def test_missing_driver_input_is_fatal(tmp_path):
    """fopen_check, as the reference's drivers use it for ibm3d.in and the
    STL, exits with the reference's message when the file is missing."""
    code = ("import ctypes, sys; sys.path.insert(0, {root!r}); import importlib; "
            "ibm = importlib.import_module('2020researchproject_gb300'); lib = ibm.load_library(); "
            "lib.fopen_check.restype = ctypes.c_void_p; "
            "lib.fopen_check(b'{path}', b'rb'); print('opened')").format(
        root=ROOT, path=os.path.join(str(tmp_path), "nope.in"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 255 and "opened" not in r.stdout
    assert 'error: cannot open file' in r.stderr
