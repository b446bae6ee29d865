"""Seeded workload generators: sizes, distributions and rod-tree topology."""
import math

import numpy as np

from boltzmannmfx_gb300 import configs
from boltzmannmfx_gb300.abi import FUNGI, YEAST


def test_sphere_plain_distributions():
    w = configs.sphere_plain()
    P = w.particles
    assert w.n == 2000 and w.steps == 100 and w.dt == 0.25
    assert (P["cell_type"] == YEAST).all()
    assert P["radius"].min() >= 5e-4 and P["radius"].max() <= 8e-4
    assert P["z"].min() >= 0.040 and P["z"].max() <= 0.052
    assert P["x"].max() < 0.128 and P["y"].max() < 0.128
    assert tuple(w.geoms[0].n_cell) == (64, 64, 32)


def test_sphere_fp32_size():
    w = configs.sphere_fp32()
    assert w.n == 200_000 and abs(w.geoms[0].prob_hi[0] - 0.512) < 1e-12 and w.steps == 500


def test_colonies_loguniform():
    w = configs.colonies()
    s = np.array(w.meta["sizes"])
    assert len(s) == 256 and s.min() >= 500 and s.max() <= 50_000
    assert 1.5e6 < s.sum() < 4.5e6
    assert np.array_equal(np.diff(w.offsets), s)


def test_rod_trees_topology():
    w = configs.rod_trees(ntrees=20, per_tree=100)
    P = w.particles
    n = P.n
    assert (P["cell_type"] == FUNGI).all()
    L = P["c_length"]
    assert L.min() >= 30e-4 and L.max() <= 35e-4
    ids = {int(v): i for i, v in enumerate(P["id"])}
    s1 = P["seg_id1"].reshape(4, n)
    st = P["site"].reshape(4, n)
    nb = P["n_bnds"]
    assert nb.max() <= 4
    for i in range(n):
        for k in range(nb[i]):
            j = ids[int(s1[k, i])]
            back = [m for m in range(nb[j]) if s1[m, j] == P["id"][i]]
            assert back, "bonds must be mutual"
            # bonded ends coincide
            def end(q, site):
                th, ph = P["theta"][q], P["phi"][q]
                u = np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])
                c = np.array([P["x"][q], P["y"][q], P["z"][q]])
                return c + (0.5 if site == 2 else -0.5) * L[q] * u
            dv = end(i, st[k, i]) - end(j, st[back[0], j])
            dv[0] -= round(dv[0] / 0.512) * 0.512
            dv[1] -= round(dv[1] / 0.512) * 0.512
            assert np.linalg.norm(dv) < 1e-12


def test_bench_cpu_samples_keep_whole_colonies():
    """The CPU arm's stratified sample: whole colonies in the workload's size
    mix, at least one even when a single colony exceeds the target."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    w = configs.sphere_fp32()
    P, g, off, take = bench.sample_colonies(w, 50_000)
    assert take == 1 and P.n == w.n and list(off) == [0, w.n]
    w = configs.colonies(ncol=24)
    P, g, off, take = bench.sample_colonies(w, w.n // 4)
    assert 1 <= take < 24 and P.n == off[-1] and len(g) == take
    sizes = np.diff(w.offsets)
    assert set(np.diff(off).tolist()) <= set(sizes.tolist())
