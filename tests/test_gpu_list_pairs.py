"""The pair set the FP32F list step (k_list_step) actually accumulates, against
the reference's gated pair set, on the 256-colony workload (2 731 333 spheres)
after list steps, and the step's force against the FP64 oracle on the same
positions.

The reference walks its full neighbour list and keeps a pair when
r^2 <= (r_lm - 1e-15)^2 (bmx_pc_interaction.cpp:212); the list step keeps it
when its FP32 offsets give r^2 < rA^2.  The two sets are equal except, at
most, for pairs whose FP64 distance lies within FP32 rounding of the cutoff
(|r - rA| <= 1e-6 rA), where the FP32 gate may decide the other way; such
pairs carry a force of order k (1e-6 rA)^2 rS.

Tolerances: pair sets exact outside that band (and the band holds at most
1e-5 of the pairs); forces within 1e-5 norm-wise relative of the FP64 oracle
(the precision form's bar)."""
import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_FP32F, Particles
from common import relerr

pytestmark = pytest.mark.gpu

TOL32 = 1e-5
BAND = 1e-6


def gated_pairs(O, prm, g, P):
    """Every candidate of the oracle's neighbour list with its distance, r_lm
    and whether the reference's gate keeps it."""
    offs, idx, img = O.pairs(prm, g, P)
    i = np.repeat(np.arange(P.n), np.diff(offs))
    L = [g.prob_hi[d] - g.prob_lo[d] for d in range(3)]
    sx = (img % 3 - 1).astype(np.float64)
    sy = (img // 3 - 1).astype(np.float64)
    # the ghost copy's position x_j + s L (FP64), then the difference
    dx = P["x"][i] - (P["x"][idx] + sx * L[0])
    dy = P["y"][i] - (P["y"][idx] + sy * L[1])
    dz = P["z"][i] - P["z"][idx]
    r = np.sqrt(dx * dx + dy * dy + dz * dz)
    assert r.max() < 4.0 * max(g.prob_hi[d] / g.n_cell[d] for d in range(3)), "image convention"
    rlm = P["radius"][i] + P["radius"][idx] + prm.bndry_width
    keep = r * r <= (rlm - 1e-15) ** 2
    return i, idx, r, rlm, keep


def compare_gated(O, prm, geoms, offsets, Q, offs, idx, colonies):
    """The step's gated pairs of the given colonies against the reference's:
    equal outside the FP32 band, none twice; returns (pairs, pairs in the band)."""
    total = band = 0
    for c in colonies:
        lo, hi = int(offsets[c]), int(offsets[c + 1])
        P = Q.subset(lo, hi)
        i, j, r, rlm, keep = gated_pairs(O, prm, geoms[c], P)
        ref = {}
        for a, b, k in zip(i.tolist(), j.tolist(), keep.tolist()):
            if k:
                ref.setdefault(a, []).append(b)
        near = {(a, b) for a, b, rr, rl in zip(i.tolist(), j.tolist(), r.tolist(), rlm.tolist())
                if abs(rr - rl) <= BAND * rl}
        for a in range(P.n):
            got = set((idx[offs[lo + a]:offs[lo + a + 1]] - lo).tolist())
            want = set(ref.get(a, []))
            assert len(got) == offs[lo + a + 1] - offs[lo + a], "a pair accumulated twice"
            diff = got ^ want
            for b in diff:
                assert (a, b) in near, (c, a, b)
            band += len(diff)
            total += len(want)
    return total, band


def test_list_cells_of_tall_short_and_narrow_boxes(gpu_lib, oracle_lib):
    """Colonies in boxes 28, 45, 70 and 32 z bins tall and of unequal x-y
    extents (the list build writes each column's cell offsets 32 z bins at a
    time), one of them empty: after list steps with builds, the step's gated
    pairs equal the reference's per colony."""
    rng = np.random.default_rng(11)
    specs = [(0.128, 0.128, 0.056, 6000), (0.064, 0.128, 0.090, 5000), (0.128, 0.128, 0.064, 0),
             (0.128, 0.064, 0.140, 7000), (0.096, 0.096, 0.064, 3000)]
    parts = [configs.sphere_colony(k, lx, ly, rng) for lx, ly, lz, k in specs]
    geoms = [configs.box_geometry(lx, ly, lz) for lx, ly, lz, k in specs]
    assert [g.n_cell[2] for g in geoms] == [28, 45, 32, 70, 32]
    P = Particles.concat(parts)
    off = np.concatenate([[0], np.cumsum([p.n for p in parts])]).astype(np.int64)
    prm = configs.deck_params()
    ctx = Context(prm, geoms)
    ctx.set_state(P, off)
    ctx.step(0.25, 40, BMXG_FP32F)
    assert 2 <= ctx.stats()["n_rebins"] < 40
    Q = P.copy()
    ctx.get_state(Q, ("x", "y", "z"))
    ctx.set_pair_capture(True)
    ctx.step(0.25, 1, BMXG_FP32F)
    offs, idx = ctx.step_pairs()
    ctx.close()
    assert offs[off[2]] == offs[off[3]]  # (the empty colony holds no pair)
    total, band = compare_gated(oracle_lib, prm, geoms, off, Q, offs, idx, [0, 1, 3, 4])
    assert total > 10_000
    assert band <= 1e-4 * total, (band, total)


def test_list_step_gated_pairs_and_forces_on_the_colonies(gpu_lib, oracle_lib):
    w = configs.colonies()
    ctx = Context(w.params, w.geoms)
    ctx.set_state(w.particles, w.offsets)
    ctx.step(w.dt, 24, BMXG_FP32F)   # list steps: builds and steps between them
    assert 1 <= ctx.stats()["n_rebins"] < 24
    Q = w.particles.copy()
    ctx.get_state(Q, ("x", "y", "z"))
    ctx.set_pair_capture(True)
    ctx.step(w.dt, 1, BMXG_FP32F)
    offs, idx = ctx.step_pairs()
    V = w.particles.copy()
    ctx.get_state(V, ("velx", "vely", "velz"))
    ctx.close()
    sizes = np.diff(w.offsets)
    order = np.argsort(sizes)
    sample = sorted(set(order[::16].tolist()) | {int(order[-1]), int(order[0])})
    total, band = compare_gated(oracle_lib, w.params, w.geoms, w.offsets, Q, offs, idx, sample)
    for c in sample:
        # the step's force on these positions against the FP64 oracle
        lo, hi = int(w.offsets[c]), int(w.offsets[c + 1])
        g = w.geoms[c]
        Pr = Q.subset(lo, hi)
        fc = oracle_lib.forces(w.params, g, Pr, oracle_lib.pairs(w.params, g, Pr), nthreads=8)
        got_v = np.stack([V["velx"][lo:hi], V["vely"][lo:hi], V["velz"][lo:hi]])
        assert relerr(got_v, fc[:3]) <= TOL32, c
    assert total > 100_000
    assert band <= 1e-5 * total, (band, total)
