"""Shared helpers for the test suite."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names(prefix=""):
    """Fixture names: the solver fixtures (no prefix), or those starting with
    `prefix` (e.g. "surface_")."""
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    if prefix:
        return [n for n in names if n.startswith(prefix)]
    return [n for n in names if not n.startswith(("surface_", "stiffness_", "dynamics_", "probe_"))]


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def rel_max(a, b):
    """max |a - b| / max |b| (max-norm relative error)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def bbox_diag(x):
    x = np.asarray(x, np.float64).reshape(-1, 3)
    return float(np.linalg.norm(x.max(0) - x.min(0)))


def elastic_from_ref(g, key):
    """Reference node forces minus the body forces it adds (gravity), pins zeroed."""
    f = g[key].astype(np.float64) - g["gravity"].astype(np.float64)
    f[g["pins"]] = 0.0
    return f
