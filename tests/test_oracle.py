"""The oracle port against the reference's own code (golden vectors made by
tests/golden/make_golden.py from oracle/_ref, the reference's force header and
loop bodies compiled verbatim), and properties of its neighbour list.  CPU only."""
import itertools
import math

import numpy as np
import pytest

from boltzmannmfx_gb300 import configs
from boltzmannmfx_gb300.abi import FUNGI, YEAST, Geometry, Particles
from common import geom_of, load, mirror, params_of, particles_of

CASES = ["sphere_plain", "rods_small", "mixed", "half_bond", "pair_test", "wall_test", "fungi_network"]
CHECK = ("x", "y", "z", "theta", "phi", "velx", "vely", "velz", "wx", "wy", "wz",
         "n_bnds", "seg_id1", "seg_id2", "site", "position", "fix_site", "dltd",
         "fuse_flag", "split_flag", "new_flag")


@pytest.mark.parametrize("case", CASES)
def test_port_matches_reference_first_step(oracle_lib, case):
    O = oracle_lib
    d = load(case)
    prm, geom, P = params_of(d), geom_of(d), particles_of(d)
    pl = O.pairs(prm, geom, P)
    for got, key in zip(pl, ("pairs_offs", "pairs_idx", "pairs_img")):
        assert np.array_equal(got, d[key]), key
    fc = O.forces(prm, geom, P, pl)
    assert np.array_equal(fc, d["fc1"])          # bit-exact
    O.update(geom, P, fc, float(d["dt"]))
    for k in CHECK:
        assert np.array_equal(P[k], d["s1_" + k]), k


@pytest.mark.parametrize("case", CASES)
def test_port_matches_reference_trajectory(oracle_lib, case):
    O = oracle_lib
    d = load(case)
    prm, geom, P = params_of(d), geom_of(d), particles_of(d)
    O.evolve(prm, [geom], [0, P.n], P, float(d["dt"]), int(d["nsteps"]))
    for k in CHECK:
        assert np.array_equal(P[k], d["sN_" + k]), k


def test_port_batched_colonies(oracle_lib):
    O = oracle_lib
    d = load("colonies_small")
    prm, geom = params_of(d), geom_of(d)
    sizes = list(d["sizes"])
    parts = []
    for c in range(len(sizes)):
        P = Particles(sizes[c])
        for k in ("x", "y", "z", "radius", "cell_type"):
            P[k] = d[f"in{c}_{k}"]
        parts.append(P)
    Q = Particles.concat(parts)
    off = np.concatenate([[0], np.cumsum(sizes)])
    O.evolve(prm, [geom] * len(sizes), off, Q, 0.25, 5)
    for c in range(len(sizes)):
        for k in ("x", "y", "z", "velx", "vely", "velz"):
            assert np.array_equal(Q[k][off[c]:off[c + 1]], d[f"out{c}_{k}"]), (c, k)


def test_port_min_distance_branches(oracle_lib):
    d = load("min_distance")
    for e, t in zip(d["e"], d["tau"]):
        assert oracle_lib.min_distance(e) == tuple(t)


def _grown_bin(x, lo, dxi, lc, hc):
    v = (x - lo) * dxi - (-1.0)
    if not v > lc:
        return lc
    if v >= hc + 1.0:
        return hc
    return int(v)


def _brute_pairs(prm, geom, P):
    """All (i, j, image) with j's (image) bin within one bin of i's, r^2 <= neighborhood,
    in AMReX's bin walk order: O(N^2) restatement for small N."""
    lo, hi, n = geom.prob_lo, geom.prob_hi, geom.n_cell
    L = [hi[d] - lo[d] for d in range(3)]
    dxi = [1.0 / (L[d] / n[d]) for d in range(3)]
    X = np.stack([P["x"], P["y"], P["z"]], 1)
    b = np.array([[_grown_bin(X[i, d], lo[d], dxi[d], 1, n[d]) for d in range(3)] for i in range(P.n)])
    ents = []  # (bin tuple, entry index, src, code, pos)
    for i in range(P.n):
        ents.append(((b[i, 0], b[i, 1], b[i, 2]), i, i, 4, X[i]))
    k = P.n
    for i in range(P.n):
        for sy, sx in itertools.product((-1, 0, 1), (-1, 0, 1)):
            if sx == 0 and sy == 0:
                continue
            if sx and not (geom.is_periodic[0] and b[i, 0] == (1 if sx > 0 else n[0])):
                continue
            if sy and not (geom.is_periodic[1] and b[i, 1] == (1 if sy > 0 else n[1])):
                continue
            g = X[i].copy()
            if sx:
                g[0] = X[i, 0] + sx * L[0]
            if sy:
                g[1] = X[i, 1] + sy * L[1]
            gb = (_grown_bin(g[0], lo[0], dxi[0], 0, n[0] + 1) if sx else b[i, 0],
                  _grown_bin(g[1], lo[1], dxi[1], 0, n[1] + 1) if sy else b[i, 1], b[i, 2])
            ents.append((gb, k, i, (sx + 1) + 3 * (sy + 1), g))
            k += 1
    ents.sort(key=lambda e: (e[0], e[1]))
    offs, idx, img = [0], [], []
    for i in range(P.n):
        for e in ents:
            if e[1] == i or any(abs(e[0][dd] - b[i, dd]) > 1 for dd in range(3)):
                continue
            dv = X[i] - e[4]
            if dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2] <= prm.neighborhood:
                idx.append(e[2])
                img.append(e[3])
        offs.append(len(idx))
    return np.array(offs), np.array(idx), np.array(img)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_pairs_equal_bruteforce_restatement(oracle_lib, seed):
    rng = np.random.default_rng(seed)
    geom = Geometry.make((0, 0, 0), (0.012, 0.010, 0.008), (6, 5, 4), (1, 1, 0))
    P = configs.sphere_colony(120, 0.012, 0.010, rng, z_band=(0.0, 0.008))
    # particles exactly on faces and corners
    P["x"][:4] = [0.0, 0.012 - 1e-17, 0.002, 0.0]
    P["y"][:4] = [0.0, 0.0, 0.010 - 1e-12, 0.004]
    prm = configs.deck_params()
    prm.neighborhood = 3.0e-5 if seed == 3 else prm.neighborhood   # non-trivial predicate
    got = oracle_lib.pairs(prm, geom, P)
    ref = _brute_pairs(prm, geom, P)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_pairs_symmetric(oracle_lib):
    w = configs.sphere_plain()
    offs, idx, img = oracle_lib.pairs(w.params, w.geoms[0], w.particles)
    fwd = set()
    for i in range(w.n):
        for t in range(offs[i], offs[i + 1]):
            fwd.add((i, int(idx[t]), int(img[t])))
    for (i, j, c) in fwd:
        assert (j, i, mirror(c)) in fwd


def test_empty_and_single(oracle_lib):
    geom = configs.box_geometry(0.128, 0.128)
    prm = configs.deck_params()
    P = Particles(0)
    offs, idx, img = oracle_lib.pairs(prm, geom, P)
    assert len(offs) == 1 and len(idx) == 0
    P = Particles(1)
    P["x"], P["y"], P["z"], P["radius"] = 0.01, 0.01, 0.047, 6e-4
    pl = oracle_lib.pairs(prm, geom, P)
    fc = oracle_lib.forces(prm, geom, P, pl)
    rA = 6e-4 + prm.z_bndry_width
    dz = 0.047 - prm.z_wall
    assert fc[2, 0] == prm.z_stiffness * rA * rA * 6e-4 - prm.z_gravity * prm.z_stiffness * rA * rA * 6e-4
    assert dz < 0


def test_analytic_sphere_law(oracle_lib):
    """F(R_S) = 0, F(R_A) = 0, repulsive inside R_S, adhesive between (cubic law
    of bmx_cell_interaction_K.H:243-276)."""
    prm = configs.deck_params()
    P = Particles(2)
    P["radius"] = [6e-4, 7e-4]
    rS = 13e-4
    rA = rS + prm.bndry_width
    for r, sign in ((rS, 0), (rA, 0), (0.9 * rS, 1), (rS + 0.5 * prm.bndry_width, -1)):
        v, w = oracle_lib.pair_force(prm, [r, 0.0, 0.0], P, 0, 1)
        if sign == 0:
            assert abs(v[0]) < 1e-25
        else:
            assert np.sign(v[0]) == sign
        assert not w.any()


def test_wall_equilibrium(oracle_lib):
    """With gravity off the sphere wall law vanishes at dz = R_S and dz >= R_A."""
    prm = configs.deck_params()
    prm.z_gravity = 0.0
    P = Particles(1)
    P["radius"] = 6e-4
    for dz, zero in ((6e-4, True), (6e-4 + prm.z_bndry_width, True), (3e-4, False), (-1e-4, False)):
        P["z"] = prm.z_wall + dz
        v, _ = oracle_lib.surface_force(prm, P, 0)
        scale = prm.z_stiffness * (6e-4 + prm.z_bndry_width) ** 2 * 6e-4
        assert (abs(v[2]) < 1e-12 * scale) == zero


def test_rod_noise_floor_is_real(oracle_lib):
    """A one-ulp change of the segment angles moves the reference's rod
    velocities by more than 1e-10 of their scale: coincident bonded ends make
    the bond force k_bond x rounding noise.  This is why the FP64 rod bar
    adds that sensitivity to the 1e-10 relative tolerance."""
    from common import trig_floor
    d = load("rods_small")
    fv, fw = trig_floor(oracle_lib, params_of(d), geom_of(d), particles_of(d))
    vmax = np.abs(d["fc1"][:3]).max()
    assert fv > 1e-11 * vmax
    assert fv < 1e-6 * vmax
