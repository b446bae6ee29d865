"""Seeded synthetic workloads for the DEM step.

The reference ships no benchmark data; its decks (exec/fungi/input_fungi,
exec/pair_test/input_pair, exec/wall_test/input_fungi) give the geometry and
force parameters, and these generators draw particles with the sizes and
distributions the five benchmark configurations name:

  sphere_plain   2 000 spheres, 0.128 x 0.128 x 0.064 cm, 100 steps (FP64 plain)
  sphere_fp32    200 000 spheres, 0.512 x 0.512 x 0.064 cm, 500 steps (FP32 pair math)
  rod_trees      50 000 rod segments in 500 branching trees, 200 steps
  colonies       256 colonies, log-uniform 500..50 000 spheres each, 200 steps
  adjoint        20 000 spheres, 200 steps (gradient checks)

Bins are the level-2 cells of the fungi deck: 0.128 cm / 64 = 0.002 cm
(exec/fungi/input_fungi:35-43 with amr.max_level = 2).
"""
import math
from dataclasses import dataclass, field

import numpy as np

from .abi import FUNGI, YEAST, Geometry, Params, Particles
from .abi import SITE_INTERIOR, SITE_SECOND_2, SITE_TIP

BIN = 0.002            # cm, level-2 cell of the fungi deck
Z_BAND = (0.040, 0.052)  # bmx.tag_region_lo/hi z of exec/fungi/input_fungi:46-47
SEED = 43343           # bmx.seed of exec/fungi/input_fungi:5
ROD_DT = 2.5e-4        # stable step for k_bond = 5e3 (see rod_trees)


def deck_params(stiffness=1.0e3, bond_strength=5.0e3):
    """cell_force.* of exec/fungi/input_fungi:148-161 and fluid.surface_location
    (:117); stiffness/bond_strength as the configurations name them.
    neighborhood = 1.1*(2*r(max_vol) + neighbor_width) (src/chemistry/bmx_chem.cpp:114-124)."""
    max_vol = 6.872e-10
    r = (3.0 * max_vol / (4.0 * math.pi)) ** (1.0 / 3.0)
    p = Params()
    p.bndry_width = 1.0e-4
    p.stiffness = stiffness
    p.z_wall = 0.048
    p.z_bndry_width = 1.0e-4
    p.z_stiffness = 1.0e5
    p.z_gravity = 0.01
    p.bond_strength = bond_strength
    p.bond_cutoff = 5.0e-4
    p.viscosity = 200.0
    p.neighborhood = 1.1 * (2.0 * r + 1.0e-2)
    return p


def box_geometry(lx, ly, lz=0.064, bin_size=BIN):
    n = [int(round(lx / bin_size)), int(round(ly / bin_size)), int(round(lz / bin_size))]
    return Geometry.make((0.0, 0.0, 0.0), (lx, ly, lz), n, (1, 1, 0))


@dataclass
class Workload:
    name: str
    params: Params
    geoms: list
    particles: Particles
    offsets: np.ndarray          # int64[ncol+1]
    dt: float
    steps: int
    precision: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def ncol(self):
        return len(self.geoms)

    @property
    def n(self):
        return self.particles.n


def sphere_colony(n, lx, ly, rng, z_band=Z_BAND, rmin=5.0e-4, rmax=8.0e-4):
    p = Particles(n)
    p["x"] = rng.uniform(0.0, lx, n)
    p["y"] = rng.uniform(0.0, ly, n)
    p["z"] = rng.uniform(z_band[0], z_band[1], n)
    r = rng.uniform(rmin, rmax, n)
    p["radius"] = r
    p["area"] = 4.0 * math.pi * r * r
    p["cell_type"] = YEAST
    return p


def spheres(name, n, lx, ly, steps, seed=SEED, precision=0, dt=0.25):
    rng = np.random.default_rng(seed)
    p = sphere_colony(n, lx, ly, rng)
    return Workload(name, deck_params(), [box_geometry(lx, ly)], p,
                    np.array([0, n], np.int64), dt, steps, precision)


def sphere_plain(seed=SEED):
    return spheres("sphere_plain_2k", 2000, 0.128, 0.128, 100, seed)


def sphere_fp32(seed=SEED, n=200_000):
    side = 0.512 * math.sqrt(n / 200_000)
    side = BIN * max(3, round(side / BIN))
    return spheres(f"sphere_fp32_{n // 1000}k", n, side, side, 500, seed, precision=1)


def colonies(seed=SEED, ncol=256, nmin=500, nmax=50_000, steps=200):
    """Independent colonies with log-uniform sizes, each in its own
    0.128 x 0.128 x 0.064 box with the plain-form distributions."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), ncol)).astype(np.int64)
    parts = [sphere_colony(int(k), 0.128, 0.128, rng) for k in sizes]
    p = Particles.concat(parts)
    p["id"] = np.arange(1, p.n + 1, dtype=np.int32)
    off = np.zeros(ncol + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    return Workload(f"colonies_{ncol}", deck_params(), [box_geometry(0.128, 0.128)] * ncol,
                    p, off, 0.25, steps, 1, meta={"sizes": sizes.tolist()})


def adjoint_spheres(seed=SEED, n=20_000):
    return spheres(f"adjoint_{n // 1000}k", n, 0.128, 0.128, 200, seed)


def _unit(theta, phi):
    st = math.sin(theta)
    return np.array([st * math.cos(phi), st * math.sin(phi), math.cos(theta)])


def rod_trees(seed=SEED, ntrees=500, per_tree=100, lx=0.512, ly=0.512,
              lmin=30.0e-4, lmax=35.0e-4, radius=2.0e-4, p_branch=0.05,
              branch_deg=(30.0, 90.0), z_band=Z_BAND):
    """Branching hyphal trees grown segment by segment: each new segment starts
    at the site-2 end of its parent (bonded ends coincide), the heading
    random-walks in phi and stays near-horizontal; with probability p_branch a
    segment also starts a side branch at an angle U(branch_deg) from its
    parent.  Bonds go into n_bnds / seg*_id1 / seg*_id2 / site* with the
    reference's site convention (site 1 at c - L/2 n, site 2 at c + L/2 n,
    bmx_cell_interaction_K.H:567-572)."""
    rng = np.random.default_rng(seed)
    n = ntrees * per_tree
    P = Particles(n, rods=True)
    X = np.zeros((n, 3))
    TH = np.zeros(n)
    PH = np.zeros(n)
    L = rng.uniform(lmin, lmax, n)
    bonds = [[] for _ in range(n)]  # (partner index, my site)
    k = 0
    zlo, zhi = z_band
    for t in range(ntrees):
        root_end = np.array([rng.uniform(0, lx), rng.uniform(0, ly), rng.uniform(zlo + 0.002, zhi - 0.002)])
        phi0 = rng.uniform(0.0, 2.0 * math.pi)
        # frontier of (parent index or -1, start point, heading theta, heading phi)
        frontier = [(-1, root_end, math.pi / 2 + rng.normal(0, 0.05), phi0)]
        start = k
        while k < start + per_tree and frontier:
            j = rng.integers(len(frontier))
            parent, end, th, ph = frontier.pop(j)
            th = min(max(th + rng.normal(0.0, 0.05), math.pi / 2 - 0.3), math.pi / 2 + 0.3)
            ph = (ph + rng.normal(0.0, 0.15)) % (2.0 * math.pi)
            u = _unit(th, ph)
            c = end + 0.5 * L[k] * u
            if c[2] < zlo + 0.001 or c[2] > zhi - 0.001:      # keep in the z band
                th = math.pi - th
                u = _unit(th, ph)
                c = end + 0.5 * L[k] * u
            X[k] = c
            TH[k] = th
            PH[k] = ph
            if parent >= 0:
                bonds[k].append((parent, 1))
                bonds[parent].append((k, 2))
            tip = c + 0.5 * L[k] * u
            frontier.append((k, tip, th, ph))
            if rng.random() < p_branch:
                ang = math.radians(rng.uniform(*branch_deg)) * (1 if rng.random() < 0.5 else -1)
                frontier.append((k, tip, th, (ph + ang) % (2.0 * math.pi)))
            k += 1
        # keep at most 4 bonds per segment (intIdx has seg1..seg4)
    assert k == n
    X[:, 0] %= lx
    X[:, 1] %= ly
    P["x"], P["y"], P["z"] = X[:, 0], X[:, 1], X[:, 2]
    P["theta"], P["phi"] = TH, PH
    P["c_length"] = L
    P["radius"] = radius
    P["area"] = 2.0 * math.pi * radius * L + 2.0 * math.pi * radius * radius
    P["cell_type"] = FUNGI
    P["cpu"] = 0
    P["bond_scale"] = 1.0
    ids = P["id"]
    nb = np.zeros(n, np.int32)
    s1 = P["seg_id1"].reshape(4, n)
    s2 = P["seg_id2"].reshape(4, n)
    st = P["site"].reshape(4, n)
    for i in range(n):
        bl = bonds[i][:4]
        nb[i] = len(bl)
        for m, (j, site) in enumerate(bl):
            s1[m, i] = ids[j]
            s2[m, i] = 0
            st[m, i] = site
    P["n_bnds"] = nb
    pos = np.full(n, SITE_INTERIOR, np.int32)
    has_child = np.zeros(n, bool)
    for i in range(n):
        for j, site in bonds[i]:
            if site == 2:
                has_child[i] = True
    pos[~has_child] = SITE_TIP
    for i in range(n):
        if has_child[i] and any((not has_child[j]) and site == 2 for j, site in bonds[i]):
            pos[i] = SITE_SECOND_2
    P["position"] = pos
    # The configuration names k_bond = 5e3 but no time step.  The explicit
    # overdamped update is stable for a bond only while
    # dt * k_bond * (d0 + db) < 2 (closing rate of two bonded ends, segment
    # mobility d0 + db ~ 0.9 at viscous_drag = 200); the plain-form
    # dt = 0.25 breaks that 400-fold and the reference trajectory leaves the
    # box within a few steps.  dt = 2.5e-4 keeps k_bond = 5e3 inside the bound.
    return Workload("rod_trees_50k" if n == 50_000 else f"rod_trees_{n}", deck_params(),
                    [box_geometry(lx, ly)], P, np.array([0, n], np.int64), ROD_DT, 200, 0)


def by_name(name, **kw):
    table = {"sphere_plain": sphere_plain, "sphere_fp32": sphere_fp32,
             "rod_trees": rod_trees, "colonies": colonies, "adjoint": adjoint_spheres}
    return table[name](**kw)
