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


def trig_floor(O, prm, geom, P):
    """How far the reference step's velocity (rows 0-2) and angular velocity
    (rows 3-5) move when every segment's angles move by one ulp -- the size
    of a last-bit difference between two libm sin/cos implementations.
    Bonded rod ends coincide, so bond forces are k_bond times the rounding
    noise of the end-point arithmetic; two correct implementations with
    different sin/cos disagree at this level.  Returns (floor_v, floor_w)."""
    pl = O.pairs(prm, geom, P)
    base = P.copy()
    fc0 = O.forces(prm, geom, base, pl)
    dv = np.zeros(6)
    for direction in (np.inf, -np.inf):
        Q = P.copy()
        Q["theta"] = np.nextafter(Q["theta"], direction)
        Q["phi"] = np.nextafter(Q["phi"], direction)
        fc = O.forces(prm, geom, Q, pl)
        dv = np.maximum(dv, np.abs(fc - fc0).max(axis=1))
    return float(dv[:3].max()), float(dv[3:].max())


def within(a, b, rel, floor):
    """max |a - b| <= rel * max |b| + floor"""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max()) <= rel * float(np.abs(b).max()) + floor
