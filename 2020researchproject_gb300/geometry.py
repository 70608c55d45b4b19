"""Synthetic inputs for the immersed-boundary fractional-step workloads.

Everything here is deterministic (seeded where random) and uses only IEEE
basic operations in numpy, so an STL or face array built on one host is
byte-identical on another.

* STL writers: an icosphere (recursive icosahedron subdivision with radial
  projection; shared vertices are written as the same float32 triple, facet
  normals are unit outward, the reader takes them from the file as the
  reference does, src/geo3d.c:251-254) and unions of axis-aligned boxes.
* Face-coordinate generators for the stretched grids: uniform, cosine bump
  clustered around a body, and the tanh wall-normal stretching
  ``y_j = tanh(beta*(2j/N - 1)) / tanh(beta)``.
"""
from __future__ import annotations

import struct

import numpy as np

__all__ = [
    "icosphere", "box_union", "write_stl", "read_stl_arrays",
    "uniform_faces", "body_clustered_faces", "tanh_faces",
]


def icosphere(subdivisions: int, radius: float = 0.5, center=(0.0, 0.0, 0.0)):
    """Return (vertices float32 [V,3], faces int [F,3]) of an icosphere.

    Faces are counter-clockwise seen from outside.  ``subdivisions=5`` gives
    20 * 4**5 = 20480 triangles.
    """
    t = (1.0 + np.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.sqrt(np.dot(v, v)) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                m = m / np.sqrt(np.dot(m, m))
                cache[key] = len(verts)
                verts.append(m)
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    v = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    v32 = v.astype(np.float32)
    f = np.array(faces, dtype=np.int64)
    # Orient every face outward (normal along centroid - center).
    c = np.asarray(center, dtype=np.float64)
    p = v32.astype(np.float64)
    n = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    out = np.einsum("ij,ij->i", n, p[f].mean(axis=1) - c) < 0
    f[out] = f[out][:, ::-1]
    return v32, f


def bumpy_sphere(subdivisions: int, radius: float = 0.5, amp: float = 0.25, center=(0.0, 0.0, 0.0)):
    """A star-shaped body with dents and bulges: the icosphere's unit
    vertices moved radially by 1 + amp (x^2 y - 0.5 z^2 x + 0.3 y z), a
    polynomial (only +, -, *), so the mesh is the same on every IEEE host.
    ``subdivisions=6`` gives 81,920 triangles, 7 gives 327,680.  Faces keep
    the sphere's outward orientation (a radial map with a positive factor
    preserves it)."""
    v, f = icosphere(subdivisions, 1.0)
    u = v.astype(np.float64)
    x, y, z = u[:, 0], u[:, 1], u[:, 2]
    fac = 1.0 + amp * (x * x * y - 0.5 * z * z * x + 0.3 * y * z)
    w = u * (radius * fac)[:, None] + np.asarray(center, dtype=np.float64)
    return w.astype(np.float32), f


def box_union(boxes):
    """Triangulate axis-aligned boxes ``[(lo(3), hi(3)), ...]`` (12 triangles
    each, outward CCW).  Boxes must not overlap or touch: the reference's
    topology walk needs every shell to be a closed 2-manifold."""
    vs, fs = [], []
    quads = [  # corner indices (bit0=x, bit1=y, bit2=z), CCW seen from inside
        (0, 2, 6, 4), (1, 5, 7, 3),   # -x, +x
        (0, 4, 5, 1), (2, 3, 7, 6),   # -y, +y
        (0, 1, 3, 2), (4, 6, 7, 5),   # -z, +z
    ]
    for lo, hi in boxes:
        lo = np.asarray(lo, dtype=np.float64)
        hi = np.asarray(hi, dtype=np.float64)
        base = len(vs)
        for c in range(8):
            vs.append([hi[0] if c & 1 else lo[0], hi[1] if c & 2 else lo[1], hi[2] if c & 4 else lo[2]])
        for a, b, c, d in quads:
            fs.append((base + a, base + c, base + b))
            fs.append((base + a, base + d, base + c))
    return np.array(vs, dtype=np.float32), np.array(fs, dtype=np.int64)


def write_stl(path, vertices, faces):
    """Write a binary STL with unit facet normals computed from the float32
    vertex coordinates."""
    v = np.asarray(vertices, dtype=np.float32)
    f = np.asarray(faces, dtype=np.int64)
    p = v.astype(np.float64)
    n = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    n = n / np.sqrt(np.einsum("ij,ij->i", n, n))[:, None]
    rec = np.zeros(len(f), dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    rec["n"] = n.astype(np.float32)
    rec["v"] = v[f]
    with open(path, "wb") as fh:
        fh.write(b"ibm3d-gb300 synthetic body".ljust(80, b" "))
        fh.write(struct.pack("<I", len(f)))
        fh.write(rec.tobytes())


def read_stl_arrays(path):
    """Return (normals [F,3] float32, triangles [F,3,3] float32)."""
    with open(path, "rb") as fh:
        data = fh.read()
    n = struct.unpack("<I", data[80:84])[0]
    rec = np.frombuffer(data[84:84 + 50 * n],
                        dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    return rec["n"].copy(), rec["v"].copy()


def uniform_faces(lo: float, hi: float, n: int) -> np.ndarray:
    """Face coordinates lo + (hi-lo)*i/n, as ``xf[i] = (double)i / N`` in the
    reference's cavity driver (src/cavity.c:28-36) when lo=0, hi=1."""
    i = np.arange(n + 1, dtype=np.float64)
    return lo + (hi - lo) * (i / n)


def body_clustered_faces(lo: float, hi: float, n: int, center: float = 0.0,
                         half_width: float = 3.0, amp: float = 4.0) -> np.ndarray:
    """Faces whose density is 1 + amp*(1+cos(pi*(x-center)/half_width))/2
    inside |x-center| < half_width and 1 outside: cells are (1+amp) times
    finer at the body than far away.  The cumulative density is inverted by
    bisection, so the result is exactly reproducible."""
    def cdf(x):
        s = x - lo
        a = np.clip(lo, center - half_width, center + half_width)
        b = np.clip(x, center - half_width, center + half_width)
        ua = (a - center) / half_width
        ub = (b - center) / half_width
        bump = amp * 0.5 * ((b - a) + half_width / np.pi * (np.sin(np.pi * ub) - np.sin(np.pi * ua)))
        return s + bump
    total = cdf(np.float64(hi))
    targets = total * (np.arange(n + 1, dtype=np.float64) / n)
    a = np.full(n + 1, lo, dtype=np.float64)
    b = np.full(n + 1, hi, dtype=np.float64)
    for _ in range(200):
        m = 0.5 * (a + b)
        below = cdf(m) < targets
        a = np.where(below, m, a)
        b = np.where(below, b, m)
    x = 0.5 * (a + b)
    x[0], x[-1] = lo, hi
    return x


def tanh_faces(n: int, beta: float = 2.0, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """Wall-normal faces y_j = tanh(beta*(2j/n - 1))/tanh(beta), mapped to [lo, hi]."""
    j = np.arange(n + 1, dtype=np.float64)
    y = np.tanh(beta * (2.0 * j / n - 1.0)) / np.tanh(beta)
    y[0], y[-1] = -1.0, 1.0
    return lo + (hi - lo) * (y + 1.0) / 2.0
