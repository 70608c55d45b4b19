"""Shared test helpers.  Marker ``gpu``: needs a CUDA device (GB300)."""
import importlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def package():
    return importlib.import_module("2020researchproject_gb300")


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["meta"] = json.loads(str(out["meta"]))
    return out


def case_stl(meta):
    """Path of a golden case's body: a committed STL next to the fixtures,
    or, for "stl_gen" cases (meshes too large to commit), the same mesh
    regenerated into the temporary directory (deterministic: only +, -, *,
    / and sqrt, so it is the mesh the fixture was made with)."""
    if "stl_gen" not in meta:
        return os.path.join(GOLDEN, meta["stl"])
    import tempfile
    gen = meta["stl_gen"]
    path = os.path.join(tempfile.gettempdir(), f"ibm3d_golden_{gen}.stl")
    if not os.path.exists(path):
        geometry = importlib.import_module("2020researchproject_gb300.geometry")
        assert gen.startswith("bumpy"), gen
        tmp = path + f".{os.getpid()}"
        geometry.write_stl(tmp, *geometry.bumpy_sphere(int(gen[5:])))
        os.replace(tmp, path)
    return path


def rel_l2(a, b, mask=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if mask is None:
        mask = np.isfinite(b)
    d = a[mask] - b[mask]
    nb = np.linalg.norm(b[mask])
    return float(np.linalg.norm(d) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="session")
def ibm():
    return package()
