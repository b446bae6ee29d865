"""Helpers shared by the tests: golden fixtures -> particles / params / geometry,
and norm-wise relative errors."""
import os

import numpy as np

from boltzmannmfx_gb300.abi import PLANE_FIELDS, Geometry, Params, Particles

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def params_of(d):
    p = Params()
    for (k, _), v in zip(Params._fields_, d["params"]):
        setattr(p, k, float(v))
    return p


def geom_of(d):
    return Geometry.make(d["lo"], d["hi"], d["n_cell"], d["periodic"])


def particles_of(d, prefix="in_"):
    n = len(d[prefix + "x"])
    P = Particles(n, rods=bool((d[prefix + "cell_type"] == 1).any()))
    for k in P.a:
        if prefix + k in d:
            P.a[k][...] = d[prefix + k]
    return P


def relerr(a, b):
    """max |a - b| / max |b| over the whole field (norm-wise, as the forms are judged)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    s = np.abs(b).max() if b.size else 0.0
    if s == 0.0:
        return float(np.abs(a - b).max()) if a.size else 0.0
    return float(np.abs(a - b).max() / s)


def same_pairs(p, q):
    return all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(p, q))


def mirror(img):
    """image code of the reverse pair: (sx, sy) -> (-sx, -sy)"""
    sx = img % 3 - 1
    sy = img // 3 - 1
    return (1 - sx) + 3 * (1 - sy)
