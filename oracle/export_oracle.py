"""CPU restatement of the reference's result export (TEST INFRASTRUCTURE
ONLY: used by tests/ as the checker of the GPU export, never by the
product package).

src/ibm3d_export.c:71-79 copies the FP64 fields into float arrays indexed
[k][j][i] over the padded grid (indices 0 .. N+3); :110-141 computes, for
each padded cell, central differences clamped to that range,

    d(f)/dx = (f[inext] - f[iprev]) / (x[inext] - x[iprev])

with the difference taken in float, the division in double and the result
stored as float, then |curl u| (float products and sums, square root in
double) and Q = dudx dvdy + dvdy dwdz + dwdz dudx - dudy dvdx - dvdz dwdy
- dudz dwdx evaluated left to right in float.  The reference is built
with -O3 and without -ffast-math on x86-64 (no contraction), so every
operation is one IEEE rounding and numpy's float32 element-wise
arithmetic reproduces it.

Parity: the reference's export needs netCDF and MPI and is not built
here, so this restatement is pinned by known answers instead (linear
velocity fields, whose clamped differences are exact) in
tests/test_export_host.py.
"""
import numpy as np


def to_file_layout(f):
    """Solver layout [i][j][k] (FP64) -> file layout [k][j][i] (float32),
    src/ibm3d_export.c:71-79."""
    return np.ascontiguousarray(np.asarray(f, dtype=np.float64).transpose(2, 1, 0)).astype(np.float32)


def _grad(f, c, axis):
    """Clamped central difference of float32 field f (layout [k][j][i])
    along `axis` (2: x, 1: y, 0: z), coordinates c (double, padded)."""
    n = f.shape[axis]
    idx = np.arange(n)
    prev = np.maximum(idx - 1, 0)
    nxt = np.minimum(idx + 1, n - 1)
    df = np.take(f, nxt, axis=axis) - np.take(f, prev, axis=axis)          # float32
    c = np.asarray(c, dtype=np.float64)
    dc = c[nxt] - c[prev]
    shape = [1, 1, 1]
    shape[axis] = n
    return (df.astype(np.float64) / dc.reshape(shape)).astype(np.float32)


def vorticity_q(u, v, w, x, y, z):
    """u, v, w: float32 [k][j][i]; x, y, z: padded centroids (double).
    Returns (|curl u|, Q) as float32, src/ibm3d_export.c:110-141."""
    u, v, w = (np.asarray(a, dtype=np.float32) for a in (u, v, w))
    dudx, dudy, dudz = _grad(u, x, 2), _grad(u, y, 1), _grad(u, z, 0)
    dvdx, dvdy, dvdz = _grad(v, x, 2), _grad(v, y, 1), _grad(v, z, 0)
    dwdx, dwdy, dwdz = _grad(w, x, 2), _grad(w, y, 1), _grad(w, z, 0)
    ox = dwdy - dvdz
    oy = dudz - dwdx
    oz = dvdx - dudy
    s2 = (ox * ox + oy * oy) + oz * oz
    vort = np.sqrt(s2.astype(np.float64)).astype(np.float32)
    q = dudx * dvdy + dvdy * dwdz
    q = q + dwdz * dudx
    q = q - dudy * dvdx
    q = q - dvdz * dwdy
    q = q - dudz * dwdx
    return vort, q
