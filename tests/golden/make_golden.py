"""Generate the golden vectors under tests/golden/ from the reference's own code.

Run in a checkout that has the reference tree (default /root/reference, or
$BMX_REFERENCE): it builds oracle/_ref/libbmxref.so -- the reference's force
header and the two loop bodies of src/des/bmx_pc_interaction.cpp compiled
verbatim -- and records its forces, positions and integer side effects for
seeded inputs.  Neighbour lists come from the oracle port (AMReX, which builds
them in the reference, is not in the reference tree).

Cases:
  sphere_plain   2 000 spheres of the plain-form configuration, 1 and 20 steps
  rods_small     400 rod segments in 10 branching trees, 1 and 20 steps (rod
                 cases use the stable rod step configs.ROD_DT)
  mixed          spheres and rods in one state
  half_bond      rods with a one-sided bond and a SECOND_2 segment (bookkeeping)
  pair_test      the two spheres across the periodic x face of exec/pair_test
                 (abc_pair_input.dat is in an older ellipsoid format; its
                 positions, radii, area and volume are read as such)
  wall_test      the single tilted rod of exec/wall_test (fungi_init_cfg.dat,
                 deck input_fungi), 100 steps
  colonies_small 4 colonies of uneven size, each stepped on its own
  min_distance   segment pairs hitting every branch of evaluateMinimumDistance
  init_bonds     InitBonds (bmx_pc_interaction.cpp:500-626 + fixBonds) on 400
                 rod segments with their bond tables cleared, a few tables
                 holding an unrelated bond first, and 100 spheres mixed in
  exchange       ParticleExchange (bmx_pc_xchng.cpp:122-151 + bmx_chem_K.H) on the
                 network below with seeded concentrations, a gentle and a
                 clamping mass-transfer rate
  split_cells    split_particles (bmx_split_particles.cpp:47-54, :90-159 +
                 checkSplit / setNewCell) on 96 AoS records, YEAST cells around
                 max_vol with FUNGI interior segments mixed in, seeded draws
  split_fungi    the same on 160 hyphal segments in every state checkSplit
                 looks at (tips, segments behind tips, isolated segments),
                 YEAST cells mixed in: tip extension, two-way tip split, side
                 branch, halving (setNewSegment, setNewSegments)
  fungi_network  the 410-segment hyphal network of the reference's checkpoint
                 exec/fungi/chk357900 (level 2, read with bmxg_read_checkpoint),
                 deck exec/fungi/input_fungi, 5 steps at the stable rod step
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from boltzmannmfx_gb300 import configs  # noqa: E402
from boltzmannmfx_gb300.abi import FUNGI, YEAST, Geometry, Params, Particles  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("BMX_REFERENCE", "/root/reference")


def deck(path):
    kv = {}
    for line in open(path):
        line = line.split("#")[0].strip()
        if "=" in line:
            k, v = line.split("=", 1)
            kv[k.strip()] = v.split()
    return kv


def params_from_deck(kv, neighbor_width=1.0e-2):
    p = Params()
    g = lambda k, d: float(kv[k][0]) if k in kv else d  # noqa: E731
    p.bndry_width = g("cell_force.boundary_width", 0.0)
    p.stiffness = g("cell_force.stiffness", 0.0)
    p.z_wall = g("fluid.surface_location", 0.0)
    p.z_bndry_width = g("cell_force.wall_boundary_width", 0.0)
    p.z_stiffness = g("cell_force.wall_stiffness", 0.0)
    p.z_gravity = g("cell_force.gravity", 0.0)
    p.bond_strength = g("cell_force.bond_strength", 5.0)
    p.bond_cutoff = g("cell_force.bond_cutoff", 1.0e-5)
    p.viscosity = g("cell_force.viscous_drag", 20.0)
    max_vol = g("chem_species.max_vol", 1.0e-12)
    r = (3.0 * max_vol / (4.0 * math.pi)) ** (1.0 / 3.0)
    p.neighborhood = 1.1 * (2.0 * r + g("cell_force.neighbor_width", neighbor_width))
    return p


def geom_from_deck(kv):
    lo = [float(v) for v in kv["geometry.prob_lo"]]
    hi = [float(v) for v in kv["geometry.prob_hi"]]
    ref = 2 ** int(kv["amr.max_level"][0])
    n = [int(v) * ref for v in kv["amr.n_cell"]]
    per = [int(v) for v in kv["geometry.is_periodic"]]
    return Geometry.make(lo, hi, n, per)


def pvec(p):
    return np.array([getattr(p, k) for k, _ in Params._fields_])


def run_case(name, params, geom, P, dt, nsteps, extra=None):
    """Record the reference's step on P: pairs + forces + state after step 1 and
    after nsteps (each step re-lists neighbours with the oracle port)."""
    out = {"params": pvec(params), "lo": np.array(geom.prob_lo), "hi": np.array(geom.prob_hi),
           "n_cell": np.array(geom.n_cell), "periodic": np.array(geom.is_periodic),
           "dt": np.array(dt), "nsteps": np.array(nsteps)}
    for k, v in P.a.items():
        out["in_" + k] = v.copy()
    Q = P.copy()
    for s in range(nsteps):
        pl = O.pairs(params, geom, Q)
        fc = O.forces(params, geom, Q, pl, use_ref=True)
        O.update(geom, Q, fc, dt, use_ref=True)
        if s == 0:
            out["pairs_offs"], out["pairs_idx"], out["pairs_img"] = pl
            out["fc1"] = fc.copy()
            for k, v in Q.a.items():
                out["s1_" + k] = v.copy()
    out["fcN"] = fc.copy()
    for k, v in Q.a.items():
        out["sN_" + k] = v.copy()
    if extra:
        out.update(extra)
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: n={P.n} pairs={len(out['pairs_idx'])} -> {os.path.getsize(path) // 1024} KB")


def sphere_plain():
    w = configs.sphere_plain()
    run_case("sphere_plain", w.params, w.geoms[0], w.particles, w.dt, 20)


def rods_small():
    w = configs.rod_trees(ntrees=10, per_tree=40, lx=0.064, ly=0.064)
    run_case("rods_small", w.params, w.geoms[0], w.particles, w.dt, 20)


def mixed():
    rng = np.random.default_rng(7)
    w = configs.rod_trees(seed=11, ntrees=4, per_tree=30, lx=0.032, ly=0.032)
    R = w.particles
    S = configs.sphere_colony(150, 0.032, 0.032, rng)
    S["id"] = np.arange(R.n + 1, R.n + S.n + 1, dtype=np.int32)
    P = Particles.concat([R, S])
    P.rods = True
    run_case("mixed", w.params, configs.box_geometry(0.032, 0.032), P, configs.ROD_DT, 10)


def half_bond():
    w = configs.rod_trees(seed=5, ntrees=3, per_tree=25, lx=0.032, ly=0.032)
    P = w.particles
    n = P.n
    nb = P["n_bnds"]
    s1 = P["seg_id1"].reshape(4, n)
    # drop the last bond entry of a few segments so that only the partner
    # remembers it; mark one segment SECOND_1 / fix_site to exercise the site rule
    cut = [i for i in range(n) if nb[i] >= 2][:6]
    for i in cut:
        nb[i] -= 1
        s1[nb[i], i] = 0
    P["fix_site"][cut[0]] = 2
    P["position"][cut[1]] = 1
    run_case("half_bond", w.params, w.geoms[0], P, configs.ROD_DT, 3)


def pair_test():
    kv = deck(os.path.join(REF, "exec/pair_test/input_pair"))
    prm = params_from_deck(kv)
    geom = geom_from_deck(kv)
    rows = [l.split() for l in open(os.path.join(REF, "exec/pair_test/abc_pair_input.dat"))][1:]
    P = Particles(len(rows))
    for i, r in enumerate(rows):
        v = [float(t) for t in r]
        P["x"][i], P["y"][i], P["z"][i] = v[0], v[1], v[2]
        P["radius"][i] = v[3]
        P["area"][i] = v[9]
    P["cell_type"] = YEAST
    dt = float(kv["bmx.fixed_dt"][0])
    run_case("pair_test", prm, geom, P, dt, int(kv["bmx.max_step"][0]))


def wall_test():
    kv = deck(os.path.join(REF, "exec/wall_test/input_fungi"))
    prm = params_from_deck(kv)
    geom = geom_from_deck(kv)
    rows = [l.split() for l in open(os.path.join(REF, "exec/wall_test/fungi_init_cfg.dat"))][1:]
    P = Particles(len(rows), rods=True)
    names = ["x", "y", "z", "radius", "c_length", "theta", "phi", "area"]
    for i, r in enumerate(rows):
        for k, f in enumerate(names):
            P[f][i] = float(r[k])
        P["cell_type"][i] = int(r[26])
    dt = float(kv["bmx.fixed_dt"][0])
    run_case("wall_test", prm, geom, P, dt, int(kv["bmx.max_step"][0]))


def colonies_small():
    rng = np.random.default_rng(3)
    sizes = [50, 400, 1200, 137]
    parts = [configs.sphere_colony(k, 0.128, 0.128, rng) for k in sizes]
    prm = configs.deck_params()
    geom = configs.box_geometry(0.128, 0.128)
    out = {"sizes": np.array(sizes)}
    for c, P in enumerate(parts):
        Q = P.copy()
        for _ in range(5):
            pl = O.pairs(prm, geom, Q)
            fc = O.forces(prm, geom, Q, pl, use_ref=True)
            O.update(geom, Q, fc, 0.25, use_ref=True)
        for k in ("x", "y", "z", "radius", "cell_type"):
            out[f"in{c}_{k}"] = P[k].copy()
        for k in ("x", "y", "z", "velx", "vely", "velz"):
            out[f"out{c}_{k}"] = Q[k].copy()
    out["params"] = pvec(prm)
    out["lo"], out["hi"] = np.array(geom.prob_lo), np.array(geom.prob_hi)
    out["n_cell"], out["periodic"] = np.array(geom.n_cell), np.array(geom.is_periodic)
    np.savez_compressed(os.path.join(OUT, "colonies_small.npz"), **out)
    print("colonies_small:", sizes)


def min_distance():
    rng = np.random.default_rng(19)
    cases = []
    for _ in range(300):  # generic
        cases.append(rng.normal(size=12))
    for _ in range(100):  # parallel and anti-parallel (det == 0 exactly)
        a = rng.normal(size=3)
        d = rng.normal(size=3)
        off = rng.normal(size=3)
        s = float(rng.choice([-2.0, -1.0, 0.5, 1.0, 2.0]))
        cases.append(np.concatenate([a, a + d, a + off, a + off + s * d]))
    for _ in range(100):  # perpendicular (Aij == 0 exactly)
        cases.append(np.array([0, 0, 0, 1, 0, 0, rng.normal(), rng.normal(), rng.normal(),
                               0, 0, 0], float))
        cases[-1][9:12] = cases[-1][6:9] + np.array([0.0, rng.normal(), rng.normal()])
    for _ in range(100):  # near-parallel, intersecting, touching end points
        a = rng.normal(size=3)
        d = rng.normal(size=3)
        e = d + 1e-7 * rng.normal(size=3)
        cases.append(np.concatenate([a, a + d, a + 0.3 * d, a + 0.3 * d + e]))
    E = np.array(cases, np.float64)
    T = np.array([O.min_distance(e, use_ref=True) for e in E])
    np.savez_compressed(os.path.join(OUT, "min_distance.npz"), e=E, tau=T)
    print("min_distance:", len(E))


BOND_TABLES = ("n_bnds", "seg_id1", "seg_id2", "site")


def init_bonds():
    w = configs.rod_trees(seed=21, ntrees=10, per_tree=40, lx=0.064, ly=0.064)
    R = w.particles
    for k in BOND_TABLES:
        R[k][:] = 0
    S = configs.sphere_colony(100, 0.064, 0.064, np.random.default_rng(23))
    S["id"] = np.arange(R.n + 1, R.n + S.n + 1, dtype=np.int32)
    P = Particles.concat([R, S])
    P.rods = True
    geom = configs.box_geometry(0.064, 0.064)
    pl = O.pairs(w.params, geom, P)
    # a prior, unrelated bond in the tables of segments that gain at most two
    T = P.copy()
    O.init_bonds(w.params, geom, T, pl)
    pre = [i for i in range(R.n) if T["n_bnds"][i] <= 2][::17]
    n = P.n
    for i in pre:
        P["n_bnds"][i] = 1
        P["seg_id1"][i] = 999_999
        P["seg_id2"][i] = 3
        P["site"][i] = 2
    Q = P.copy()
    added, over = O.init_bonds(w.params, geom, Q, pl)
    assert over == 0
    ref = P.copy()
    O.init_bonds(w.params, geom, ref, pl, use_ref=True)
    for k in BOND_TABLES:
        assert np.array_equal(ref[k], Q[k]), k
    out = {"params": pvec(w.params), "lo": np.array(geom.prob_lo), "hi": np.array(geom.prob_hi),
           "n_cell": np.array(geom.n_cell), "periodic": np.array(geom.is_periodic),
           "rlim": np.array(O.RLIM), "added": np.array(added)}
    for k, v in P.a.items():
        out["in_" + k] = v.copy()
    for k in BOND_TABLES:
        out["out_" + k] = ref[k].copy()
    np.savez_compressed(os.path.join(OUT, "init_bonds.npz"), **out)
    print(f"init_bonds: n={n} added={added} prior={len(pre)}")


def fungi_network():
    from boltzmannmfx_gb300.runtime import read_checkpoint
    kv = deck(os.path.join(REF, "exec/fungi/input_fungi"))
    prm = params_from_deck(kv)
    geom = geom_from_deck(kv)
    P = read_checkpoint(os.path.join(REF, "exec/fungi/chk357900/particles"), 2)
    for k in ("velx", "vely", "velz", "wx", "wy", "wz"):
        P[k][:] = 0.0
    run_case("fungi_network", prm, geom, P, configs.ROD_DT, 5)


def exchange():
    d = dict(np.load(os.path.join(OUT, "fungi_network.npz")))
    prm = Params()
    for (k, _), v in zip(Params._fields_, d["params"]):
        setattr(prm, k, float(v))
    geom = Geometry.make(d["lo"], d["hi"], d["n_cell"], d["periodic"])
    P = Particles(len(d["in_x"]), rods=True)
    for k in P.a:
        if "in_" + k in d:
            P.a[k][...] = d["in_" + k]
    rng = np.random.default_rng(29)
    conc = rng.uniform(0.0, 1.0e-3, (3, P.n))
    vol = math.pi * P["radius"] ** 2 * P["c_length"]
    pl = O.pairs(prm, geom, P)
    out = {"conc": conc, "vol": vol, "dt": np.array(0.25)}
    for name, xp in (("gentle", [1.0e-2, 2.0e-2, 5.0e-3]), ("clamped", [1.0e4, 1.0e4, 1.0e4])):
        out["xpar_" + name] = np.array(xp)
        out["out_" + name] = O.particle_exchange(geom, P, vol, conc, 0.25, xp, pl=pl, use_ref=True)
    np.savez_compressed(os.path.join(OUT, "exchange.npz"), **out)
    print("exchange:", P.n)


def split_cells():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from common import split_expected_count, split_params, split_records
    n, cap = 96, 160
    a = split_records(n, cap, 41)
    k = split_expected_count(a, n)
    draws = np.random.default_rng(43).random(2 * k)
    out = a.copy()
    rc, ns = O.split_cells(out, n, split_params(), draws=draws, use_ref=True)
    assert rc == 0 and ns == k
    np.savez_compressed(os.path.join(OUT, "split_cells.npz"), in_rec=a, out_rec=out, draws=draws,
                        n=np.array(n), num_split=np.array(ns))
    print("split_cells:", n, ns)


def split_fungi():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from common import split_fungi_records, split_params
    n, cap = 160, 480
    a = split_fungi_records(n, cap, 47)
    draws = np.random.default_rng(53).random(8 * n)
    sp = split_params(brnch_prob=0.3, split_prob=0.5)
    out = a.copy()
    rc, ns, used = O.split_cells(out, n, sp, draws=draws, use_ref=True, return_used=True)
    assert rc == 0 and ns > 0
    np.savez_compressed(os.path.join(OUT, "split_fungi.npz"), in_rec=a, out_rec=out, draws=draws[:used],
                        n=np.array(n), num_split=np.array(ns),
                        params=np.array([sp.brnch_prob, sp.split_prob, sp.split_len]))
    print("split_fungi:", n, ns, used)


if __name__ == "__main__":
    O.build(ref=True)
    if not O.have_ref():
        sys.exit("reference harness not built (reference tree missing?)")
    for f in (sphere_plain, rods_small, mixed, half_bond, pair_test, wall_test, colonies_small, min_distance,
              init_bonds, fungi_network, exchange, split_cells, split_fungi):
        f()
