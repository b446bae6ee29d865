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


# cell division inputs --------------------------------------------------------

SPLIT_MAX_VOL = 5.0e-10  # SPECIES::max_vol of the size the yeast decks use (m^3)


def split_params(**kw):
    """bmxg_split_params of BMX's defaults: overlap 0.2, 3 species (9 reals
    past first_data), no extra ints; FUNGI limits, split probability and split
    length of bmx_chem_species_parms.cpp; no side branching unless asked."""
    from boltzmannmfx_gb300.abi import SplitParams
    sp = SplitParams(max_vol=SPLIT_MAX_VOL, overlap=0.2, max_len=0.0035, max_rad=0.00025,
                     brnch_prob=0.0, split_prob=0.1, split_len=0.0030, num_reals=9, num_ints=0)
    for k, v in kw.items():
        setattr(sp, k, v)
    return sp


def split_records(n, cap, seed, frac_divide=0.3, frac_fungi=0.2):
    """Seeded AoS records (abi.aos_dtype(34, 35)): YEAST cells with volumes
    around max_vol (about frac_divide of them above it), radius, area from the
    volume, every other real and int filled with seeded values so that the
    copy is checked whole, FUNGI interior segments mixed in (they never
    divide), and the daughter slots [n, cap) filled with a sentinel pattern."""
    from boltzmannmfx_gb300.abi import FUNGI, INT_IDX as I, REAL_IDX as R, YEAST, aos_dtype
    rng = np.random.default_rng(seed)
    a = np.zeros(cap, aos_dtype())
    a["pos"][:n] = rng.uniform(-1.0e-3, 1.0e-3, (n, 3))
    a["rdata"][:n] = rng.normal(0.0, 1.0, (n, 34))
    a["idata"][:n] = rng.integers(-1000, 1000, (n, 35))
    vol = SPLIT_MAX_VOL * np.where(rng.random(n) < frac_divide, rng.uniform(1.0001, 1.9, n),
                                   rng.uniform(0.4, 1.0, n))
    r = (3.0 * vol / (4.0 * np.pi)) ** (1.0 / 3.0)
    a["rdata"][:n, R["vol"]] = vol
    a["rdata"][:n, R["radius"]] = r
    a["rdata"][:n, R["area"]] = 4.0 * np.pi * r * r
    a["rdata"][:n, R["dvdt"]] = rng.uniform(0.0, 1.0e-12, n)
    fungi = rng.random(n) < frac_fungi
    a["idata"][:n, I["cell_type"]] = np.where(fungi, FUNGI, YEAST)
    a["idata"][:n, I["position"]] = np.where(fungi, 3, rng.integers(0, 4, n))
    a["id"][:n] = np.arange(1, n + 1)
    a["cpu"][:n] = rng.integers(0, 4, n)
    a["idata"][:n, I["id"]] = a["id"][:n]
    a["idata"][:n, I["cpu"]] = a["cpu"][:n]
    a["pos"][n:] = -3.0
    a["rdata"][n:] = -7.0
    a["id"][n:] = -5
    a["cpu"][n:] = -6
    a["idata"][n:] = -9
    return a


def split_expected_count(a, n, max_vol=SPLIT_MAX_VOL):
    from boltzmannmfx_gb300.abi import INT_IDX as I, REAL_IDX as R, YEAST
    return int(np.count_nonzero((a["idata"][:n, I["cell_type"]] == YEAST) & (a["rdata"][:n, R["vol"]] > max_vol)))


def split_fungi_records(n, cap, seed, frac_yeast=0.25):
    """Seeded AoS records of hyphal segments in every state checkSplit looks at:
    tips (isolated, with one or two bonds) at and below the length and radius
    limits, segments behind a tip (SECOND_1 / SECOND_2, one to three bonds),
    interior segments, and YEAST cells mixed in; every other field seeded."""
    from boltzmannmfx_gb300.abi import FUNGI, INT_IDX as I, REAL_IDX as R, YEAST
    a = split_records(n, cap, seed, frac_divide=0.3, frac_fungi=0.0)
    rng = np.random.default_rng(seed + 1000)
    fungi = rng.random(n) >= frac_yeast
    pos = rng.integers(0, 4, n)
    nb = np.where(pos == 0, rng.integers(0, 3, n), np.where(pos == 3, 2, rng.integers(1, 4, n)))
    L = np.where(rng.random(n) < 0.6, rng.uniform(0.0035, 0.0045, n), rng.uniform(0.0025, 0.0035, n))
    rad = np.where(rng.random(n) < 0.7, rng.uniform(0.00025, 0.0003, n), rng.uniform(0.0002, 0.00025, n))
    a["idata"][:n, I["cell_type"]] = np.where(fungi, FUNGI, YEAST)
    sel = np.flatnonzero(fungi)
    a["idata"][sel, I["position"]] = pos[sel]
    a["idata"][sel, I["n_bnds"]] = nb[sel]
    a["idata"][sel, 15] = rng.integers(1, 3, sel.size)          # site1
    a["rdata"][sel, R["c_length"]] = L[sel]
    a["rdata"][sel, R["radius"]] = rad[sel]
    a["rdata"][sel, R["theta"]] = rng.uniform(0.05, np.pi - 0.05, sel.size)
    a["rdata"][sel, R["phi"]] = rng.uniform(0.0, 2.0 * np.pi, sel.size)
    a["rdata"][sel, R["vol"]] = np.pi * rad[sel] ** 2 * L[sel]
    return a
