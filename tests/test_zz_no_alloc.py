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
    ibm = package()
    fn = _noalloc(ibm.load_library())
    poly = ibm.Polyhedron(os.path.join(GOLDEN, "sphere_sub2.stl"))
    x = np.linspace(-1.7, 2.3, 23)
    y = np.linspace(-1.4, 1.5, 19)
    z = np.linspace(-1.3, 1.3, 17) ** 3 * 0.6 + np.linspace(-1.3, 1.3, 17) * 0.4
    ref = poly.cpt(x, y, z)                       # Polyhedron_cpt, allocating
    assert np.isfinite(ref).all() and (ref < 0).any() and (ref > 0).any()
    for call in range(2):                         # two calls share the scratch array
        out = np.full(ref.shape, -7.0)
        rc = fn(poly._p, len(x), len(y), len(z), _p(x), _p(y), _p(z), _p(out), 15.0)
        assert rc == 0, f"call {call} failed"
        assert np.array_equal(out, ref), f"call {call}: {int((out != ref).sum())} points differ"


def test_noalloc_cpt_rejects_grids_beyond_its_buffer():
    ibm = package()
    fn = _noalloc(ibm.load_library())
    poly = ibm.Polyhedron(os.path.join(GOLDEN, "sphere_sub2.stl"))
    x = np.linspace(-2, 2, 180)
    out = np.full((180, 180, 180), 3.0)
    rc = fn(poly._p, 180, 180, 180, _p(x), _p(x), _p(x), _p(out), 15.0)
    assert rc == -1
    assert (out == 3.0).all()
