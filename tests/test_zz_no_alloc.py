"""Polyhedron_cpt_noalloc: the level-set entry point for callers that cannot
allocate device memory (a framework allocator owning the GPU,
allocation-free loops).  It must give exactly what the
allocating entry point Polyhedron_cpt gives, on consecutive calls that share
its static scratch array, and refuse grids larger than that array.

This file is collected last on purpose."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, package

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    fn = lib.Polyhedron_cpt_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]
    return fn


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_noalloc_cpt_matches_allocating_entry_point():
    """Consecutive calls that share the scratch array, on different bodies
    and differently shaped grids: each must equal Polyhedron_cpt bit for
    bit.  The second call's grid is smaller than the first and its body
    (a box) differs, so contents left from the first call (geometry,
    fallback list, output) would show."""
    ibm = package()
    fn = _noalloc(ibm.load_library())
    sphere = ibm.Polyhedron(os.path.join(GOLDEN, "sphere_sub2.stl"))
    box = ibm.Polyhedron(os.path.join(GOLDEN, "box.stl"))
    zs = np.linspace(-1.3, 1.3, 17)
    grids = [
        (sphere, np.linspace(-1.7, 2.3, 23), np.linspace(-1.4, 1.5, 19), zs ** 3 * 0.6 + zs * 0.4),
        (box, np.linspace(-0.9, 1.1, 11), np.linspace(-1.2, 0.8, 14), np.linspace(-0.7, 0.9, 9)),
        (sphere, np.linspace(-1.7, 2.3, 23), np.linspace(-1.4, 1.5, 19), zs ** 3 * 0.6 + zs * 0.4),
    ]
    for call, (poly, x, y, z) in enumerate(grids):
        ref = poly.cpt(x, y, z)                   # Polyhedron_cpt, allocating
        assert np.isfinite(ref).all() and (ref < 0).any() and (ref > 0).any()
        out = np.full(ref.shape, -7.0)
        rc = fn(poly._p, len(x), len(y), len(z), _p(x), _p(y), _p(z), _p(out), 15.0)
        assert rc == 0, f"call {call} failed"
        assert np.array_equal(out, ref), f"call {call}: {int((out != ref).sum())} points differ"


def test_noalloc_cpt_rejects_bad_sizes():
    """Non-positive grid sizes are refused on the host, output untouched."""
    ibm = package()
    fn = _noalloc(ibm.load_library())
    poly = ibm.Polyhedron(os.path.join(GOLDEN, "sphere_sub2.stl"))
    x = np.linspace(-2, 2, 8)
    out = np.full((8, 8, 8), 3.0)
    for dims in ((0, 8, 8), (8, -3, 8), (8, 8, 0)):
        assert fn(poly._p, *dims, _p(x), _p(x), _p(x), _p(out), 15.0) == -1
    assert (out == 3.0).all()


def test_noalloc_cpt_rejects_grids_beyond_its_buffer():
    ibm = package()
    fn = _noalloc(ibm.load_library())
    poly = ibm.Polyhedron(os.path.join(GOLDEN, "sphere_sub2.stl"))
    x = np.linspace(-2, 2, 180)
    out = np.full((180, 180, 180), 3.0)
    rc = fn(poly._p, 180, 180, 180, _p(x), _p(x), _p(x), _p(out), 15.0)
    assert rc == -1
    assert (out == 3.0).all()
