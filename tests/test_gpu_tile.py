"""bmxg_step_tile: the FP64 sphere step of one tile with the caller's ghost
particles (AMReX's per-tile EvolveParticles after fillNeighbors,
bmx_pc_interaction.cpp:97-279, halo of one cell: bmx_pc.cpp:23).

A domain is cut into boxes; each box's reals are the particles whose cell is
in it, its ghosts every particle (and periodic image, shifted by a domain
length as AMReX shifts it) whose cell is in the box's one-cell halo.  The
union of the per-box results must equal the single-box step bit for bit in
FP64 -- which is itself bit-exact against the oracle
(tests/test_gpu_parity.py)."""
import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_FP64, Particles
from boltzmannmfx_gb300.runtime import BmxgError

pytestmark = pytest.mark.gpu

OUT = ("x", "y", "z", "velx", "vely", "velz")


def cell_of(x, plo, dxi, lo_c, hi_c):
    """The step's 1-based cell along one axis (bin_of): (x - plo) dxi + 1,
    clamped to [lo_c, hi_c]; None leaves it unclamped."""
    v = (x - plo) * dxi + 1.0
    b = np.floor(v).astype(np.int64)
    if lo_c is not None:
        b = np.where(v > lo_c, b, lo_c)
        b = np.where(v >= hi_c + 1.0, hi_c, b)
    return b


def workload(n=20_000, seed=5):
    rng = np.random.default_rng(seed)
    P = configs.sphere_colony(n, 0.128, 0.128, rng)
    g = configs.box_geometry(0.128, 0.128)
    return configs.deck_params(), g, P


def tile_inputs(g, P, lo, hi):
    """Reals (cell inside [lo, hi]) and ghosts (cell in the one-cell halo,
    periodic images shifted by a domain length), each in index order."""
    n = [g.n_cell[d] for d in range(3)]
    plo = [g.prob_lo[d] for d in range(3)]
    L = [g.prob_hi[d] - g.prob_lo[d] for d in range(3)]
    dxi = [1.0 / (L[d] / n[d]) for d in range(3)]
    pos = [np.asarray(P[k]) for k in "xyz"]
    own = [cell_of(pos[d], plo[d], dxi[d], 1, n[d]) for d in range(3)]
    inside = np.ones(P.n, bool)
    for d in range(3):
        inside &= (own[d] >= lo[d] + 1) & (own[d] <= hi[d] + 1)
    reals = np.flatnonzero(inside)
    gidx, gpos = [], []
    for sx in (-1, 0, 1):
        for sy in (-1, 0, 1):
            if (sx and not g.is_periodic[0]) or (sy and not g.is_periodic[1]):
                continue
            q = [pos[0] + float(sx) * L[0] if sx else pos[0], pos[1] + float(sy) * L[1] if sy else pos[1], pos[2]]
            c = [cell_of(q[0], plo[0], dxi[0], None, None) if sx else own[0],
                 cell_of(q[1], plo[1], dxi[1], None, None) if sy else own[1], own[2]]
            grown = np.ones(P.n, bool)
            tile = np.ones(P.n, bool)
            for d in range(3):
                grown &= (c[d] >= lo[d]) & (c[d] <= hi[d] + 2)
                tile &= (c[d] >= lo[d] + 1) & (c[d] <= hi[d] + 1)
            sel = np.flatnonzero(grown & ~tile)
            gidx.append(sel)
            gpos.append(np.stack([q[0][sel], q[1][sel], q[2][sel]]))
    gidx = np.concatenate(gidx)
    gpos = np.concatenate(gpos, axis=1)
    order = np.argsort(gidx, kind="stable")
    gidx, gpos = gidx[order], gpos[:, order]
    R = take(P, reals)
    G = take(P, gidx)
    G["x"], G["y"], G["z"] = gpos[0].copy(), gpos[1].copy(), gpos[2].copy()
    return reals, R, G


def take(P, idx):
    Q = Particles(len(idx))
    for k in ("x", "y", "z", "radius", "cell_type", "velx", "vely", "velz"):
        Q[k] = np.ascontiguousarray(np.asarray(P[k])[idx])
    return Q


def whole_domain_step(prm, g, P, dt):
    ctx = Context(prm, [g])
    ctx.set_state(P)
    ctx.step(dt, 1, BMXG_FP64)
    Q = P.copy()
    ctx.get_state(Q, OUT)
    ctx.close()
    return Q


@pytest.mark.parametrize("cuts", [(1, 1, 1), (2, 2, 1), (2, 2, 2), (3, 2, 1)])
def test_tiles_union_equals_whole_domain_step(gpu_lib, cuts):
    prm, g, P = workload()
    dt = 0.25
    ref = whole_domain_step(prm, g, P, dt)
    n = [g.n_cell[d] for d in range(3)]
    got = {k: np.full(P.n, np.nan) for k in OUT}
    seen = np.zeros(P.n, np.int64)
    ctx = Context(prm, [g])
    edges = [np.linspace(0, n[d], cuts[d] + 1).astype(int) for d in range(3)]
    nghost = 0
    for a in range(cuts[0]):
        for b in range(cuts[1]):
            for c in range(cuts[2]):
                lo = (edges[0][a], edges[1][b], edges[2][c])
                hi = (edges[0][a + 1] - 1, edges[1][b + 1] - 1, edges[2][c + 1] - 1)
                idx, R, G = tile_inputs(g, P, lo, hi)
                nghost += G.n
                ctx.step_tile(lo, hi, R, G, dt)
                for k in OUT:
                    got[k][idx] = R[k]
                seen[idx] += 1
    ctx.close()
    assert (seen == 1).all()
    assert nghost > 0
    for k in OUT:
        assert np.array_equal(got[k], ref[k]), k


def test_tile_rejects_reals_outside_and_non_spheres(gpu_lib):
    prm, g, P = workload(n=2_000)
    ctx = Context(prm, [g])
    idx, R, G = tile_inputs(g, P, (0, 0, 0), (31, 31, 31))
    R2 = take(P, np.arange(P.n))   # every particle as a real of the first quarter
    with pytest.raises(BmxgError):
        ctx.step_tile((0, 0, 0), (31, 31, 31), R2, G, 0.25)
    R3 = take(P, idx)
    R3["cell_type"][0] = 1          # a rod segment
    with pytest.raises(BmxgError):
        ctx.step_tile((0, 0, 0), (31, 31, 31), R3, G, 0.25)
    with pytest.raises(BmxgError):  # not a box of the domain
        ctx.step_tile((0, 0, 0), (64, 31, 31), take(P, idx), G, 0.25)
    R5 = take(P, idx)
    R5["z"][0] = np.nan             # a non-finite position comes back as an error, as from bmxg_step
    with pytest.raises(BmxgError) as e:
        ctx.step_tile((0, 0, 0), (31, 31, 31), R5, G, 0.25)
    assert "non-finite" in str(e.value)
    ctx.close()


def test_tile_on_device_arrays(gpu_lib):
    """The same tile call with every array in device memory (where = BMXG_DEVICE)."""
    import ctypes as C
    import torch
    from boltzmannmfx_gb300 import abi
    prm, g, P = workload(n=5_000)
    lo, hi = (0, 0, 0), (31, 31, 31)
    idx, R, G = tile_inputs(g, P, lo, hi)
    ctx = Context(prm, [g])
    Rh = take(P, idx)
    ctx.step_tile(lo, hi, Rh, G, 0.25)          # host arrays: the expected result
    dev = {}

    def to_dev(Q, fields):
        s = abi.ParticlesStruct()
        s.n = Q.n
        for name, ctype in abi.ParticlesStruct._fields_[1:]:
            if name in fields:
                t = torch.from_numpy(np.ascontiguousarray(Q[name])).cuda()
                dev[(id(Q), name)] = t
                setattr(s, name, C.cast(C.c_void_p(t.data_ptr()), ctype))
            else:
                setattr(s, name, ctype())
        return s

    Rd = take(P, idx)
    sr = to_dev(Rd, ("x", "y", "z", "radius", "cell_type", "velx", "vely", "velz"))
    sg = to_dev(G, ("x", "y", "z", "radius", "cell_type"))
    t = abi.Tile()
    t.lo[:] = list(lo)
    t.hi[:] = list(hi)
    rc = ctx.lib.bmxg_step_tile(ctx.h, C.byref(t), C.byref(sr), C.byref(sg), 0.25, abi.BMXG_DEVICE)
    assert rc == abi.BMXG_OK, ctx.lib.bmxg_last_error(ctx.h)
    torch.cuda.synchronize()
    for k in OUT:
        got = dev[(id(Rd), k)].cpu().numpy()
        assert np.array_equal(got, Rh[k]), k
    ctx.close()
