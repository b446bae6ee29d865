"""FP32F neighbour list with a skin (k_list.cu) through the C ABI.

The list mode must give the FP32F step of the per-step stencil path (the same
pair set, FP32 rounding aside), hand exact reference bins back to every other
consumer (FP64 steps, the pair-list export), stay out of the way where it would
not be exact, and run the same steps eagerly as inside its CUDA graphs (with
the build in a conditional node)."""
import math

import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_FP32F, BMXG_FP64, Particles
from common import relerr, same_pairs

pytestmark = pytest.mark.gpu

TOL32 = 1e-5    # FP32F form, norm-wise relative force error


def ctx_for(w, P=None, mode=1):
    ctx = Context(w.params, w.geoms)
    ctx.set_list_mode(mode)
    ctx.set_state(w.particles if P is None else P, w.offsets)
    return ctx


def read(ctx, P):
    Q = P.copy()
    for k in ("velx", "vely", "velz"):
        Q[k] = np.nan
    ctx.get_state(Q)
    return Q


def vel(Q):
    return np.stack([Q["velx"], Q["vely"], Q["velz"]])


def periodic_disp(A, P, L):
    d = A - P
    return (d + L / 2) % L - L / 2


def test_list_step_matches_stencil_path(gpu_lib, oracle_lib):
    w = configs.sphere_fp32(n=40_000)
    g = w.geoms[0]
    A, B = ctx_for(w, mode=1), ctx_for(w, mode=0)
    A.step(w.dt, 1, BMXG_FP32F)
    B.step(w.dt, 1, BMXG_FP32F)
    Pr = w.particles.copy()
    fc = oracle_lib.forces(w.params, g, Pr, oracle_lib.pairs(w.params, g, Pr), nthreads=8)
    assert relerr(vel(read(A, w.particles)), fc[:3]) <= TOL32
    assert relerr(vel(read(A, w.particles)), vel(read(B, w.particles))) <= TOL32
    A.step(w.dt, 39, BMXG_FP32F)
    B.step(w.dt, 39, BMXG_FP32F)
    sa, sb = A.stats(), B.stats()
    assert 1 <= sa["n_rebins"] < 40 and sb["n_rebins"] == 40
    QA, QB = read(A, w.particles), read(B, w.particles)
    L = g.prob_hi[0] - g.prob_lo[0]
    for k in ("x", "y"):
        assert relerr(periodic_disp(QA[k], w.particles[k], L), periodic_disp(QB[k], w.particles[k], L)) <= 1e-4
    assert relerr(QA["z"] - w.particles["z"], QB["z"] - w.particles["z"]) <= 1e-4
    assert relerr(vel(QA), vel(QB)) <= 1e-4


def test_exact_bins_after_list_steps(gpu_lib, oracle_lib):
    """After list steps the pair export and an FP64 step are bit-exact to the
    oracle on the positions the list steps produced."""
    w = configs.sphere_fp32(n=40_000)
    g = w.geoms[0]
    ctx = ctx_for(w)
    ctx.step(w.dt, 21, BMXG_FP32F)
    P1 = read(ctx, w.particles)
    assert same_pairs(ctx.pairs(), oracle_lib.pairs(w.params, g, P1))
    Pr = P1.copy()
    oracle_lib.step(w.params, g, Pr, w.dt, nthreads=8)
    ctx.step(w.dt, 1, BMXG_FP64)
    Q = read(ctx, w.particles)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(Q[k], Pr[k]), k
    # and back to list steps from the FP64 state
    ctx.step(w.dt, 3, BMXG_FP32F)
    assert np.isfinite(read(ctx, w.particles)["x"]).all()


def test_graph_and_eager_steps_agree(gpu_lib):
    """The conditional-node graphs and the eager gated launches run the same
    steps: bit-identical states."""
    w = configs.sphere_fp32(n=20_000)
    A, B = ctx_for(w), ctx_for(w)
    B.set_profiling(True)   # every step eager
    l0 = A.stats()["n_kernel_launches"]
    A.step(w.dt, 24, BMXG_FP32F)
    sa = A.stats()
    B.step(w.dt, 24, BMXG_FP32F)
    sb = B.stats()
    # two kernels per step, twelve per build, and the list's set-up (the
    # fixed-point positions) once
    assert sa["n_kernel_launches"] - l0 == 2 * 24 + 12 * sa["n_rebins"] + 1
    assert sa["n_rebins"] == sb["n_rebins"]
    QA, QB = read(A, w.particles), read(B, w.particles)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(QA[k], QB[k]), k


def test_list_overflow_walks_the_stencil(gpu_lib, oracle_lib):
    """A particle with more list entries than the capacity falls back to a
    stencil walk; its force is still the reference's."""
    rng = np.random.default_rng(5)
    lx = 0.032
    bg = configs.sphere_colony(400, lx, lx, rng)
    k = 60
    c = np.array([0.016, 0.016, 0.046])
    u = rng.normal(size=(k, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    pts = c + u * rng.uniform(2e-4, 9e-4, size=(k, 1))
    cl = Particles(k)
    cl["x"], cl["y"], cl["z"] = pts[:, 0], pts[:, 1], pts[:, 2]
    cl["radius"] = 5.0e-4
    cl["area"] = 4.0 * math.pi * 5.0e-4 ** 2
    P = Particles.concat([bg, cl])
    prm = configs.deck_params()
    g = configs.box_geometry(lx, lx)
    w = configs.Workload("cluster", prm, [g], P, np.array([0, P.n], np.int64), 0.25, 1)
    A = ctx_for(w)
    A.step(w.dt, 1, BMXG_FP32F)
    Pr = P.copy()
    fc = oracle_lib.forces(prm, g, Pr, oracle_lib.pairs(prm, g, Pr))
    assert relerr(vel(read(A, P)), fc[:3]) <= TOL32


def test_list_off_where_not_exact(gpu_lib):
    """Radii whose cutoff reaches past a bin keep the per-step stencil path:
    both modes give bit-identical results and re-bin every step."""
    rng = np.random.default_rng(9)
    P = configs.sphere_colony(3000, 0.064, 0.064, rng, rmin=9.0e-4, rmax=9.6e-4)
    prm = configs.deck_params()
    g = configs.box_geometry(0.064, 0.064)
    w = configs.Workload("big", prm, [g], P, np.array([0, P.n], np.int64), 0.25, 5)
    A, B = ctx_for(w, mode=1), ctx_for(w, mode=0)
    A.step(w.dt, 5, BMXG_FP32F)
    B.step(w.dt, 5, BMXG_FP32F)
    assert A.stats()["n_rebins"] == 5
    QA, QB = read(A, P), read(B, P)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(QA[k], QB[k]), k


def test_list_batched_colonies(gpu_lib, oracle_lib):
    """Several colonies of uneven size: first-step forces against the FP64
    oracle per colony, and agreement with the stencil path over 30 steps."""
    rng = np.random.default_rng(3)
    sizes = [50, 4000, 12000, 137]
    parts = [configs.sphere_colony(k, 0.128, 0.128, rng) for k in sizes]
    P = Particles.concat(parts)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    prm = configs.deck_params()
    g = configs.box_geometry(0.128, 0.128)
    w = configs.Workload("cols", prm, [g] * len(sizes), P, off, 0.25, 30)
    A, B = ctx_for(w, mode=1), ctx_for(w, mode=0)
    A.step(w.dt, 1, BMXG_FP32F)
    QA = read(A, P)
    for c, Pc in enumerate(parts):
        fc = oracle_lib.forces(prm, g, Pc.copy(), oracle_lib.pairs(prm, g, Pc))
        assert relerr(vel(QA)[:, off[c]:off[c + 1]], fc[:3]) <= TOL32, c
    B.step(w.dt, 1, BMXG_FP32F)
    A.step(w.dt, 29, BMXG_FP32F)
    B.step(w.dt, 29, BMXG_FP32F)
    QA, QB = read(A, P), read(B, P)
    assert relerr(vel(QA), vel(QB)) <= 1e-4
    assert relerr(QA["z"] - P["z"], QB["z"] - P["z"]) <= 1e-4


def test_list_position_accumulation(gpu_lib):
    """The list path accumulates positions in 64-bit fixed point: after 24 list
    steps a position equals its start plus the sum of the steps' FP32
    increments float(dt) * v, summed in extended precision, within 4 FP64 ulp
    plus 16 fixed-point units (the conversions in and out, and the ~1e-19 cm
    of each increment's scaling to units); modulo the box in the periodic x
    and y."""
    w = configs.sphere_fp32(n=40_000)
    g = w.geoms[0]
    ctx = ctx_for(w)
    ctx.step(w.dt, 2, BMXG_FP32F)   # builds the list (a first call of one step runs the per-step path)
    P0 = read(ctx, w.particles)
    acc = {k: P0[k].astype(np.longdouble) for k in ("x", "y", "z")}
    dtf = np.float32(w.dt)
    for s in range(24):
        ctx.step(w.dt, 1, BMXG_FP32F)
        Q = read(ctx, w.particles)
        for k, v in (("x", "velx"), ("y", "vely"), ("z", "velz")):
            acc[k] += (dtf * Q[v].astype(np.float32)).astype(np.longdouble)
    assert ctx.stats()["n_rebins"] < 26
    for d, k in enumerate(("x", "y", "z")):
        want = acc[k]
        if g.is_periodic[d]:
            L = np.longdouble(g.prob_hi[d] - g.prob_lo[d])
            want = want - L * np.floor((want - np.longdouble(g.prob_lo[d])) / L)
        diff = np.abs(Q[k].astype(np.longdouble) - want)
        if g.is_periodic[d]:
            diff = np.minimum(diff, np.abs(diff - L))
        ulp = np.spacing(np.abs(Q[k]))
        # near 0 the FP64 ulp is finer than a fixed-point unit (span / 2^64)
        span = (g.prob_hi[d] - g.prob_lo[d]) * (1.0 if g.is_periodic[d] else 4.0)
        tol = 4 * ulp + 16 * np.ldexp(span, -64)
        assert np.all(diff <= tol), (k, float((diff / tol).max()))


def test_per_step_position_accumulation_is_binary64(gpu_lib):
    """The per-step FP32F path (a one-step call right after a load) accumulates
    positions in FP64: the result equals x + double(float(dt) * v) bit for bit
    (v the step's FP32 velocity)."""
    w = configs.sphere_fp32(n=40_000)
    g = w.geoms[0]
    ctx = ctx_for(w)
    ctx.step(w.dt, 1, BMXG_FP32F)
    Q = read(ctx, w.particles)
    dtf = np.float32(w.dt)
    for k, v in (("x", "velx"), ("y", "vely"), ("z", "velz")):
        inc = (dtf * Q[v].astype(np.float32)).astype(np.float64)
        want = w.particles[k] + inc
        ax = {"x": 0, "y": 1, "z": 2}[k]
        inside = (want >= g.prob_lo[ax]) & (want < g.prob_hi[ax])  # not wrapped this step
        assert inside.mean() > 0.99
        assert np.array_equal(Q[k][inside], want[inside]), k


def test_autotune_list_shapes_leave_state_and_steps_unchanged(gpu_lib, tmp_path):
    """bmxg_autotune sweeps the list step's block and passes and the build's
    block: it leaves the loaded state as it was, the steps after it are
    bit-identical to those of an untuned context (each slot's arithmetic does
    not depend on the launch shape), and a second context takes the shapes
    from the cache."""
    w = configs.colonies(ncol=12)
    cache = str(tmp_path / "tune.json")
    A, B = ctx_for(w), ctx_for(w)
    A.autotune(cache)
    sh = A.shapes()
    assert sh["list_step_block"] in (64, 128, 256) and sh["list_step_passes"] in (1, 2, 4, 8)
    assert sh["list_build_block"] in (64, 128, 256)
    Q0 = read(A, w.particles)
    for k in ("x", "y", "z"):
        assert np.array_equal(Q0[k], w.particles[k]), k
    A.step(w.dt, 24, BMXG_FP32F)
    B.step(w.dt, 24, BMXG_FP32F)
    assert A.stats()["n_rebins"] == B.stats()["n_rebins"] >= 1
    QA, QB = read(A, w.particles), read(B, w.particles)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(QA[k], QB[k]), k
    C = ctx_for(w)
    C.autotune(cache)
    assert C.shapes() == sh
    for c in (A, B, C):
        c.close()


def test_prepare_instantiates_graphs_and_changes_no_result(gpu_lib):
    """bmxg_prepare captures the step graphs without stepping: the state is
    unchanged, and the steps after it are bit-identical to those of a context
    that captured them on first use (FP32F list path and FP64)."""
    w = configs.sphere_fp32(n=20_000)
    A, B = ctx_for(w), ctx_for(w)
    A.prepare(w.dt, BMXG_FP32F)
    Q0 = read(A, w.particles)
    for k in ("x", "y", "z"):
        assert np.array_equal(Q0[k], w.particles[k]), k
    for prec in (BMXG_FP32F, BMXG_FP64):
        if prec == BMXG_FP64:
            for c in (A, B):
                c.set_state(w.particles, w.offsets)
            A.prepare(w.dt, prec)
        A.step(w.dt, 20, prec)
        B.step(w.dt, 20, prec)
        QA, QB = read(A, w.particles), read(B, w.particles)
        for k in ("x", "y", "z", "velx", "vely", "velz"):
            assert np.array_equal(QA[k], QB[k]), (prec, k)
    A.close()
    B.close()


def test_prepare_rods_fp32f_pipeline(gpu_lib):
    """bmxg_prepare on a rod state allocates the FP32F rod pipeline and captures
    its graphs: the steps after it equal those of an unprepared context."""
    w = configs.rod_trees(ntrees=40, per_tree=50)
    A, B = Context(w.params, w.geoms), Context(w.params, w.geoms)
    for c in (A, B):
        c.set_state(w.particles, w.offsets)
    A.prepare(w.dt, BMXG_FP32F)
    for c in (A, B):
        c.step(w.dt, 20, BMXG_FP32F)
    QA, QB = w.particles.copy(), w.particles.copy()
    A.get_state(QA)
    B.get_state(QB)
    for k in ("x", "y", "z", "theta", "phi", "velx", "vely", "velz", "wx", "wy", "wz"):
        assert np.array_equal(QA[k], QB[k]), k
    A.close()
    B.close()


@pytest.mark.parametrize("shape", [dict(list_step_persistent=True, list_step_passes=4),
                                   dict(list_step_persistent=True, list_step_block=64, list_step_passes=8),
                                   dict(list_step_block=256, list_step_passes=1, list_build_block=64)])
def test_list_shapes_bitwise_same_steps(gpu_lib, shape):
    """Every launch shape of the list step and build (one block per chunk, or
    one persistent wave taking chunks from a counter) gives bit-identical
    steps, the persistent dispenser resetting itself between launches."""
    w = configs.colonies(ncol=12)
    A, B = ctx_for(w), ctx_for(w)
    A.set_shapes(**shape)
    for c in (A, B):
        c.step(w.dt, 24, BMXG_FP32F)
        c.step(w.dt, 5, BMXG_FP32F)  # eager steps after the graph replays
    assert A.stats()["n_rebins"] == B.stats()["n_rebins"] >= 1
    QA, QB = read(A, w.particles), read(B, w.particles)
    for k in ("x", "y", "z", "velx", "vely", "velz"):
        assert np.array_equal(QA[k], QB[k]), k
    with pytest.raises(Exception):
        A.set_shapes(list_step_block=48)
    A.close()
    B.close()
