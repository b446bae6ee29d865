"""InitBonds (src/des/bmx_pc_interaction.cpp:500-626 with fixBonds,
src/chemistry/bmx_cell_interaction_K.H:1287-1440): the oracle port against the
golden tables made by the reference's own loop body, and the GPU kernel
through the C ABI against the same tables."""
import math

import numpy as np
import pytest

from boltzmannmfx_gb300 import configs
from boltzmannmfx_gb300.abi import FUNGI, BMXG_ERR_CAPACITY, Particles
from common import geom_of, load, params_of, particles_of

TABLES = ("n_bnds", "seg_id1", "seg_id2", "site")


def test_port_matches_golden(oracle_lib):
    d = load("init_bonds")
    P = particles_of(d)
    added, over = oracle_lib.init_bonds(params_of(d), geom_of(d), P, rlim=float(d["rlim"]))
    assert over == 0
    assert added == int(d["added"])
    for k in TABLES:
        assert np.array_equal(P[k], d["out_" + k]), k


def test_port_matches_reference_harness(oracle_lib):
    """Live comparison with the reference's loop body where it is built here."""
    if not oracle_lib.have_ref():
        pytest.skip("reference harness not built")
    w = configs.rod_trees(seed=9, ntrees=6, per_tree=30, lx=0.032, ly=0.032)
    P = w.particles
    for k in TABLES:
        P[k][:] = 0
    pl = oracle_lib.pairs(w.params, w.geoms[0], P)
    A, B = P.copy(), P.copy()
    oracle_lib.init_bonds(w.params, w.geoms[0], A, pl)
    oracle_lib.init_bonds(w.params, w.geoms[0], B, pl, use_ref=True)
    for k in TABLES:
        assert np.array_equal(A[k], B[k]), k


def star(nseg=6, L=3.0e-3, r=2.0e-4):
    """nseg segments whose site-1 ends all sit at one point: each meets
    nseg - 1 others there, more than the four table slots when nseg > 5."""
    P = Particles(nseg, rods=True)
    c = np.array([0.016, 0.016, 0.046])
    for k in range(nseg):
        ph = 2.0 * math.pi * k / nseg
        u = np.array([math.cos(ph), math.sin(ph), 0.0])
        x = c + 0.5 * L * u
        P["x"][k], P["y"][k], P["z"][k] = x
        P["theta"][k] = 0.5 * math.pi
        P["phi"][k] = ph
    P["c_length"] = L
    P["radius"] = r
    P["area"] = 2.0 * math.pi * r * L + 2.0 * math.pi * r * r
    P["cell_type"] = FUNGI
    P["id"] = np.arange(1, nseg + 1, dtype=np.int32)
    P["bond_scale"] = 1.0
    return P


def test_port_overflow_counted(oracle_lib):
    P = star(6)
    prm = configs.deck_params()
    g = configs.box_geometry(0.032, 0.032)
    added, over = oracle_lib.init_bonds(prm, g, P)
    assert added == 6 * 4 and over == 6
    assert (P["n_bnds"] == 4).all()
    # each table lists four of the others, with this segment's site 1
    s1 = P["seg_id1"].reshape(4, -1)
    for i in range(6):
        assert set(s1[:, i]) <= set(range(1, 7)) - {i + 1}
    assert (P["site"].reshape(4, -1) == 1).all()


def test_port_no_fungi_pairs(oracle_lib):
    """Spheres never bond; an empty state is a no-op."""
    prm = configs.deck_params()
    g = configs.box_geometry(0.032, 0.032)
    S = configs.sphere_colony(50, 0.032, 0.032, np.random.default_rng(1))
    Q = Particles(S.n, rods=True)
    for k in S.a:
        Q[k] = S[k]
    assert oracle_lib.init_bonds(prm, g, Q) == (0, 0)
    E = Particles(0, rods=True)
    assert oracle_lib.init_bonds(prm, g, E) == (0, 0)


@pytest.mark.gpu
def test_gpu_matches_golden(gpu_lib):
    from boltzmannmfx_gb300.runtime import Context
    d = load("init_bonds")
    P = particles_of(d)
    ctx = Context(params_of(d), [geom_of(d)])
    ctx.set_state(P)
    added, over = ctx.init_bonds(float(d["rlim"]))
    assert (added, over) == (int(d["added"]), 0)
    Q = P.copy()
    ctx.get_state(Q)
    for k in TABLES:
        assert np.array_equal(Q[k], d["out_" + k]), k


@pytest.mark.gpu
def test_gpu_then_step_matches_port(gpu_lib, oracle_lib):
    """Bonds found on the GPU drive the next step like the port's do."""
    from boltzmannmfx_gb300.abi import BMXG_FP64
    from boltzmannmfx_gb300.runtime import Context
    d = load("init_bonds")
    P = particles_of(d)
    prm, g = params_of(d), geom_of(d)
    ref = P.copy()
    oracle_lib.init_bonds(prm, g, ref)
    ctx = Context(prm, [g])
    ctx.set_state(P)
    ctx.init_bonds()
    ctx.step(configs.ROD_DT, 1, BMXG_FP64)
    Q = P.copy()
    ctx.get_state(Q)
    oracle_lib.step(prm, g, ref, configs.ROD_DT)
    for k in TABLES + ("position",):
        assert np.array_equal(Q[k], ref[k]), k


@pytest.mark.gpu
def test_gpu_overflow_status(gpu_lib):
    from boltzmannmfx_gb300.runtime import BmxgError, Context
    P = star(6)
    ctx = Context(configs.deck_params(), [configs.box_geometry(0.032, 0.032)])
    ctx.set_state(P)
    with pytest.raises(BmxgError) as e:
        ctx.init_bonds()
    assert e.value.code == BMXG_ERR_CAPACITY
    Q = P.copy()
    ctx.get_state(Q)
    assert (Q["n_bnds"] == 4).all()
