"""CUDA product (libbmxg.so through the C ABI) against the oracle and the
golden vectors of the reference's own code.

Bars: neighbour lists bit-exact in every form; the FP64 sphere step
bit-exact; the FP64 rod step within 1e-10 norm-wise relative (the kernel
applies the segment mobility once per segment instead of once per pair, which
reorders the rounding); the FP32F form within 1e-5 norm-wise relative force
error against FP64."""
import math

import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_FP32F, BMXG_FP64, Particles
from common import geom_of, load, params_of, particles_of, relerr, same_pairs, trig_floor, within

pytestmark = pytest.mark.gpu

TOL64 = 1e-10   # FP64 rod path, norm-wise relative
TOL32 = 1e-5    # FP32F form, norm-wise relative force error

OUT_FIELDS = ("x", "y", "z", "theta", "phi", "velx", "vely", "velz", "wx", "wy", "wz")
INT_FIELDS = ("n_bnds", "seg_id1", "seg_id2", "site", "position", "fix_site", "dltd",
              "fuse_flag", "split_flag", "new_flag")


def gpu_ctx(prm, geoms, P, offsets=None):
    ctx = Context(prm, geoms)
    ctx.set_state(P, offsets)
    return ctx


def readback(ctx, P):
    Q = P.copy()
    for k in ("velx", "vely", "velz", "wx", "wy", "wz"):
        Q[k] = np.nan
    ctx.get_state(Q)
    return Q


@pytest.mark.parametrize("case", ["sphere_plain", "pair_test", "rods_small", "mixed", "half_bond", "wall_test",
                                  "fungi_network"])
def test_pairs_bitexact_golden(gpu_lib, case):
    d = load(case)
    ctx = gpu_ctx(params_of(d), [geom_of(d)], particles_of(d))
    got = ctx.pairs()
    assert same_pairs(got, (d["pairs_offs"], d["pairs_idx"], d["pairs_img"]))


@pytest.mark.parametrize("case", ["sphere_plain", "pair_test"])
def test_sphere_fp64_bitexact_golden(gpu_lib, case):
    d = load(case)
    P = particles_of(d)
    ctx = gpu_ctx(params_of(d), [geom_of(d)], P)
    ctx.step(float(d["dt"]), 1, BMXG_FP64)
    Q = readback(ctx, P)
    assert np.array_equal(Q["velx"], d["fc1"][0])
    assert np.array_equal(Q["vely"], d["fc1"][1])
    assert np.array_equal(Q["velz"], d["fc1"][2])
    for k in ("x", "y", "z"):
        assert np.array_equal(Q[k], d["s1_" + k]), k
    ctx.step(float(d["dt"]), int(d["nsteps"]) - 1, BMXG_FP64)
    Q = readback(ctx, P)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(Q[k], d["sN_" + k]), k


@pytest.mark.parametrize("case", ["rods_small", "mixed", "half_bond", "wall_test", "fungi_network"])
def test_rod_fp64_golden(gpu_lib, oracle_lib, case):
    """Within 1e-10 of the field's scale, plus the reference's own sensitivity
    to a one-ulp change of the segment angles (trig_floor): CUDA's and glibc's
    sin/cos may differ in the last bit, and bond forces on coincident ends
    are k_bond times end-point rounding noise."""
    d = load(case)
    P = particles_of(d)
    prm, g = params_of(d), geom_of(d)
    fv, fw = trig_floor(oracle_lib, prm, g, P)
    ctx = gpu_ctx(prm, [g], P)
    ctx.step(float(d["dt"]), 1, BMXG_FP64)
    Q = readback(ctx, P)
    fc = np.stack([Q[k] for k in ("velx", "vely", "velz", "wx", "wy", "wz")])
    assert within(fc[:3], d["fc1"][:3], TOL64, 8 * fv)
    assert within(fc[3:], d["fc1"][3:], TOL64, 8 * fw)
    for k in ("x", "y", "z", "theta", "phi"):
        assert relerr(Q[k], d["s1_" + k]) <= TOL64, k
    for k in INT_FIELDS:
        assert np.array_equal(Q[k], d["s1_" + k]), k
    ctx.step(float(d["dt"]), int(d["nsteps"]) - 1, BMXG_FP64)
    Q = readback(ctx, P)
    for k in ("x", "y", "z", "theta", "phi"):
        assert relerr(Q[k], d["sN_" + k]) <= TOL64, k
    for k in INT_FIELDS:
        assert np.array_equal(Q[k], d["sN_" + k]), k


def test_colonies_batched_golden(gpu_lib):
    d = load("colonies_small")
    sizes = list(d["sizes"])
    parts = []
    for c in range(len(sizes)):
        P = Particles(sizes[c])
        for k in ("x", "y", "z", "radius", "cell_type"):
            P[k] = d[f"in{c}_{k}"]
        parts.append(P)
    Q = Particles.concat(parts)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    ctx = gpu_ctx(params_of(d), [geom_of(d)] * len(sizes), Q, off)
    ctx.step(0.25, 5, BMXG_FP64)
    R = readback(ctx, Q)
    for c in range(len(sizes)):
        for k in ("x", "y", "z", "velx", "vely", "velz"):
            assert np.array_equal(R[k][off[c]:off[c + 1]], d[f"out{c}_{k}"]), (c, k)


def test_full_size_sphere_fp32_config(gpu_lib, oracle_lib):
    """200 000 spheres: pair list bit-exact, FP64 step bit-exact, FP32F force
    error <= 1e-5 against the FP64 oracle."""
    O = oracle_lib
    w = configs.sphere_fp32()
    g = w.geoms[0]
    P = w.particles
    ctx = gpu_ctx(w.params, [g], P)
    ref_pairs = O.pairs(w.params, g, P)
    assert same_pairs(ctx.pairs(), ref_pairs)
    Pr = P.copy()
    fc = O.forces(w.params, g, Pr, ref_pairs, nthreads=8)
    O.update(g, Pr, fc, w.dt, nthreads=8)
    ctx.step(w.dt, 1, BMXG_FP64)
    Q = readback(ctx, P)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(Q[k], Pr[k]), k
    ctx.set_state(P)
    ctx.step(w.dt, 1, BMXG_FP32F)
    Q = readback(ctx, P)
    v32 = np.stack([Q["velx"], Q["vely"], Q["velz"]])
    assert relerr(v32, fc[:3]) <= TOL32
    assert same_pairs(ctx.pairs(), O.pairs(w.params, g, Q))


def test_fp32f_rods_error(gpu_lib, oracle_lib):
    O = oracle_lib
    w = configs.rod_trees(ntrees=40, per_tree=100)
    g = w.geoms[0]
    P = w.particles
    Pr = P.copy()
    pl = O.pairs(w.params, g, Pr)
    fc = O.forces(w.params, g, Pr, pl, nthreads=8)
    ctx = gpu_ctx(w.params, [g], P)
    assert same_pairs(ctx.pairs(), pl)
    ctx.step(w.dt, 1, BMXG_FP32F)
    Q = readback(ctx, P)
    got = np.stack([Q[k] for k in ("velx", "vely", "velz", "wx", "wy", "wz")])
    assert relerr(got[:3], fc[:3]) <= TOL32
    assert relerr(got[3:], fc[3:]) <= TOL32


def test_trajectory_long_fp64_spheres(gpu_lib, oracle_lib):
    """100 steps of the 2 000-sphere plain configuration, bit-exact to the oracle."""
    w = configs.sphere_plain()
    Pr = w.particles.copy()
    oracle_lib.evolve(w.params, w.geoms, [0, w.n], Pr, w.dt, w.steps)
    ctx = gpu_ctx(w.params, w.geoms, w.particles)
    ctx.step(w.dt, w.steps, BMXG_FP64)
    Q = readback(ctx, w.particles)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(Q[k], Pr[k]), k
    assert same_pairs(ctx.pairs(), oracle_lib.pairs(w.params, w.geoms[0], Pr))


def test_evolve_particles_dropin(gpu_lib):
    w = configs.sphere_plain()
    ctx = gpu_ctx(w.params, w.geoms, w.particles)
    cost, nsub = ctx.evolve_particles(w.dt)
    assert nsub == 1 and cost == [float(w.n)]


def test_fp32f_multistep_bins_stay_exact(gpu_lib, oracle_lib):
    """50 FP32F steps (several FP32-offset re-sync periods): the neighbour list
    of the resulting FP64 positions is still exactly the reference's, and the
    displacements follow the FP64 trajectory."""
    w = configs.sphere_fp32(n=40_000)
    g = w.geoms[0]
    ctx32 = gpu_ctx(w.params, [g], w.particles)
    ctx64 = gpu_ctx(w.params, [g], w.particles)
    ctx32.step(w.dt, 50, BMXG_FP32F)
    ctx64.step(w.dt, 50, BMXG_FP64)
    A = readback(ctx32, w.particles)
    B = readback(ctx64, w.particles)
    assert same_pairs(ctx32.pairs(), oracle_lib.pairs(w.params, g, A))
    L = g.prob_hi[0] - g.prob_lo[0]
    for k in ("x", "y", "z"):
        da = A[k] - w.particles[k]
        db = B[k] - w.particles[k]
        if k != "z":  # periodic wrap: compare displacements modulo the box
            da = (da + L / 2) % L - L / 2
            db = (db + L / 2) % L - L / 2
        assert relerr(da, db) <= 1e-4, k
    v32 = np.stack([A["velx"], A["vely"], A["velz"]])
    v64 = np.stack([B["velx"], B["vely"], B["velz"]])
    assert relerr(v32, v64) <= 1e-4


def test_full_size_colonies(gpu_lib, oracle_lib):
    """The benchmark's 256-colony workload at full size (2 731 333 spheres):
    one FP64 step bit-exact against the oracle; the FP32F force error of a list
    step within 1e-5 of the FP64 step's; 24 FP32F list steps against 24 per-step
    FP32F steps within 1e-4 in the displacements; and after the list steps the
    exported pair list equals that of a fresh exact binning of the positions."""
    import os
    w = configs.colonies()
    P = w.particles
    A = gpu_ctx(w.params, w.geoms, P, w.offsets)
    A.step(w.dt, 1, BMXG_FP64)
    Q64 = readback(A, P)
    R = P.copy()
    oracle_lib.evolve(w.params, w.geoms, w.offsets, R, w.dt, 1, nthreads=os.cpu_count() or 1)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(Q64[k], R[k]), k
    # a list step (build + step) and an FP64 step on the same positions
    A.set_state(P, w.offsets)
    A.step(w.dt, 1, BMXG_FP64)
    A.step(w.dt, 1, BMXG_FP32F)
    assert A.stats()["n_rebins"] == 2   # the FP64 step's binning and one list build
    C = gpu_ctx(w.params, w.geoms, P, w.offsets)
    C.step(w.dt, 2, BMXG_FP64)
    va = np.stack([readback(A, P)[k] for k in ("velx", "vely", "velz")])
    vc = np.stack([readback(C, P)[k] for k in ("velx", "vely", "velz")])
    assert relerr(va, vc) <= TOL32
    # list steps against per-step FP32F steps
    A.set_state(P, w.offsets)
    A.step(w.dt, 24, BMXG_FP32F)
    D = Context(w.params, w.geoms)
    D.set_list_mode(0)
    D.set_state(P, w.offsets)
    D.step(w.dt, 24, BMXG_FP32F)
    QA, QD = readback(A, P), readback(D, P)
    assert A.stats()["n_rebins"] < 24 and D.stats()["n_rebins"] == 24
    L = 0.128
    for k in ("x", "y"):
        da = QA[k] - P[k] - L * np.round((QA[k] - P[k]) / L)
        dd = QD[k] - P[k] - L * np.round((QD[k] - P[k]) / L)
        assert relerr(da, dd) <= 1e-4, k
    assert relerr(QA["z"] - P["z"], QD["z"] - P["z"]) <= 1e-4
    # the pair list after list steps is the exact binning's
    E = gpu_ctx(w.params, w.geoms, QA, w.offsets)
    assert same_pairs(A.pairs(), E.pairs())
