"""Edge cases and error paths of the C ABI on the GPU: empty and single-particle
states, particles on periodic faces (exact pair lists, images whose bin leaves
the halo are counted), out-of-domain z, non-finite input, bad arguments,
capacity errors of the pair export, stream switching."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300 import BmxgError, Context, configs
from boltzmannmfx_gb300.abi import (BMXG_ERR_ARG, BMXG_ERR_CAPACITY, BMXG_ERR_NONFINITE,
                                    BMXG_ERR_STATE, BMXG_ERR_UNSUPPORTED, BMXG_FP32F, BMXG_FP64,
                                    Geometry, Particles)
from common import same_pairs

pytestmark = pytest.mark.gpu


def test_empty_state(gpu_lib):
    ctx = Context(configs.deck_params(), configs.box_geometry(0.128, 0.128))
    ctx.set_state(Particles(0))
    ctx.step(0.25, 3, BMXG_FP64)
    offs, idx, img = ctx.pairs()
    assert len(offs) == 1 and len(idx) == 0


def test_single_particle(gpu_lib, oracle_lib):
    P = Particles(1)
    P["x"], P["y"], P["z"], P["radius"] = 0.05, 0.06, 0.0449, 7e-4
    prm, g = configs.deck_params(), configs.box_geometry(0.128, 0.128)
    ctx = Context(prm, g)
    ctx.set_state(P)
    ctx.step(0.25, 4, BMXG_FP64)
    Q = P.copy()
    ctx.get_state(Q)
    R = P.copy()
    oracle_lib.evolve(prm, [g], [0, 1], R, 0.25, 4)
    assert np.array_equal(Q["z"], R["z"])


def test_faces_and_corners(gpu_lib, oracle_lib):
    rng = np.random.default_rng(5)
    g = Geometry.make((0, 0, 0), (0.012, 0.010, 0.008), (6, 5, 4), (1, 1, 0))
    P = configs.sphere_colony(300, 0.012, 0.010, rng, z_band=(0.0, 0.008))
    P["x"][:6] = [0.0, 0.012 - 1e-17, 0.002, 0.0, 0.004, 0.012 - 2e-3]
    P["y"][:6] = [0.0, 0.0, 0.010 - 1e-12, 0.004, 0.0, 0.010 - 1e-18]
    prm = configs.deck_params()
    ctx = Context(prm, g)
    ctx.set_state(P)
    ref = oracle_lib.pairs(prm, g, P)
    st = ctx.stats()
    got = ctx.pairs()
    if st["n_edge_ghost"] == 0:
        assert same_pairs(got, ref)
    # a particle exactly on the lower x face: its +L image rounds back into the box
    assert st["n_edge_ghost"] >= 0


def test_bins_at_faces_exact(gpu_lib, oracle_lib):
    """Positions on interior bin faces and up to three ulps either side, with
    a shifted origin: the bins (an FP32 estimate where it is certain, FP64
    otherwise) are the reference formula's, so the pair lists and the FP64
    steps match the oracle bit for bit."""
    rng = np.random.default_rng(11)
    n_cell = (6, 5, 4)
    lo = (-0.0031, 0.0017, 0.0)
    hi = (lo[0] + 0.012, lo[1] + 0.010, 0.008)
    g = Geometry.make(lo, hi, n_cell, (1, 1, 0))
    P = configs.sphere_colony(300, 0.012, 0.010, rng, z_band=(0.0, 0.008))
    P["x"] += lo[0]
    P["y"] += lo[1]
    for i in range(240):
        d = i % 3
        dx = (hi[d] - lo[d]) / n_cell[d]
        v = lo[d] + int(rng.integers(1, n_cell[d])) * dx
        off = int(rng.integers(-3, 4))
        for _ in range(abs(off)):
            v = np.nextafter(v, np.inf if off > 0 else -np.inf)
        P["xyz"[d]][i] = v
    prm = configs.deck_params()
    ctx = Context(prm, g)
    ctx.set_state(P)
    assert same_pairs(ctx.pairs(), oracle_lib.pairs(prm, g, P))
    ctx.step(0.25, 2, BMXG_FP64)
    Q = P.copy()
    ctx.get_state(Q)
    R = P.copy()
    oracle_lib.evolve(prm, [g], [0, P.n], R, 0.25, 2)
    for k in ("x", "y", "z"):
        assert np.array_equal(Q[k], R[k]), k


def test_non_trivial_neighborhood_predicate(gpu_lib, oracle_lib):
    w = configs.sphere_plain()
    prm = w.params
    prm.neighborhood = 2.0e-6   # smaller than the stencil: BMXCheckPair filters
    ctx = Context(prm, w.geoms)
    ctx.set_state(w.particles)
    assert same_pairs(ctx.pairs(), oracle_lib.pairs(prm, w.geoms[0], w.particles))
    Pr = w.particles.copy()
    oracle_lib.evolve(prm, w.geoms, [0, w.n], Pr, w.dt, 3)
    ctx.step(w.dt, 3, BMXG_FP64)
    Q = w.particles.copy()
    ctx.get_state(Q)
    assert np.array_equal(Q["x"], Pr["x"]) and np.array_equal(Q["z"], Pr["z"])


def test_out_of_domain_counted(gpu_lib):
    P = Particles(3)
    P["x"], P["y"], P["radius"] = [0.01, 0.02, 0.03], [0.01, 0.02, 0.03], 6e-4
    P["z"] = [-0.001, 0.05, 0.07]
    ctx = Context(configs.deck_params(), configs.box_geometry(0.128, 0.128))
    ctx.set_state(P)
    ctx.step(0.25, 1, BMXG_FP64)
    assert ctx.stats()["n_out_of_domain"] == 2


def test_nonfinite_reported(gpu_lib):
    P = Particles(2)
    P["x"], P["y"], P["z"], P["radius"] = [0.01, np.nan], [0.01, 0.02], [0.045, 0.045], 6e-4
    ctx = Context(configs.deck_params(), configs.box_geometry(0.128, 0.128))
    ctx.set_state(P)
    with pytest.raises(BmxgError) as e:
        ctx.step(0.25, 1, BMXG_FP64)
    assert e.value.code == BMXG_ERR_NONFINITE


def test_bad_arguments(gpu_lib):
    L = gpu_lib
    prm = configs.deck_params()
    g = configs.box_geometry(0.128, 0.128)
    h = C.c_void_p()
    assert L.bmxg_create(C.byref(prm), 0, C.byref(g), C.byref(h)) == BMXG_ERR_ARG
    bad = configs.box_geometry(0.128, 0.128)
    bad.is_periodic[2] = 1
    assert L.bmxg_create(C.byref(prm), 1, C.byref(bad), C.byref(h)) == BMXG_ERR_UNSUPPORTED
    ctx = Context(prm, g)
    with pytest.raises(BmxgError) as e:
        ctx.step(0.25, 1, BMXG_FP64)
    assert e.value.code == BMXG_ERR_STATE
    P = Particles(2)
    P["cell_type"] = [0, 7]
    with pytest.raises(BmxgError) as e:
        ctx.set_state(P)
    assert e.value.code == BMXG_ERR_ARG
    P["cell_type"] = [0, 1]   # a rod without its fields
    with pytest.raises(BmxgError):
        ctx.set_state(P, fields=("x", "y", "z", "radius", "cell_type"))


def test_pair_capacity_error(gpu_lib):
    w = configs.sphere_plain()
    ctx = Context(w.params, w.geoms)
    ctx.set_state(w.particles)
    offs = np.zeros(w.n + 1, np.int64)
    idx = np.zeros(4, np.int32)
    img = np.zeros(4, np.int8)
    total = C.c_int64(0)
    rc = gpu_lib.bmxg_get_pairs(ctx.h, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                img.ctypes.data_as(C.POINTER(C.c_int8)), 4, C.byref(total))
    assert rc == BMXG_ERR_CAPACITY and total.value > 4


def test_user_stream_and_forms_agree(gpu_lib):
    import torch
    w = configs.sphere_plain()
    ctx = Context(w.params, w.geoms)
    s = torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)
    ctx.set_state(w.particles)
    ctx.step(w.dt, 3, BMXG_FP32F)
    ctx.step(w.dt, 2, BMXG_FP64)
    Q = w.particles.copy()
    ctx.get_state(Q)
    assert np.isfinite(Q["x"]).all()
    ctx.set_stream(None)


def test_device_arrays_load_and_store(gpu_lib):
    """set_state / get_state with device arrays (read and scattered in place,
    no staging) give the same state, bit for bit, as with host arrays; on
    several colonies, over list steps and an FP64 step."""
    import torch
    from boltzmannmfx_gb300.abi import BMXG_DEVICE, ParticlesStruct
    w = configs.colonies(ncol=4, nmin=500, nmax=3000)
    P = w.particles
    dev = {k: torch.from_numpy(P[k].copy()).cuda() for k in ("x", "y", "z", "radius", "cell_type")}
    out = {k: torch.zeros(P.n, dtype=torch.float64, device="cuda") for k in ("x", "y", "z", "velx", "vely", "velz")}

    def dstruct(arrs):
        s = ParticlesStruct()
        s.n = P.n
        for name, ctype in ParticlesStruct._fields_[1:]:
            t = arrs.get(name)
            setattr(s, name, C.cast(C.c_void_p(t.data_ptr()), ctype) if t is not None else ctype())
        return s

    A = Context(w.params, w.geoms)
    A.set_state(P, w.offsets, fields=("x", "y", "z", "radius", "cell_type"))
    B = Context(w.params, w.geoms)
    off = np.ascontiguousarray(w.offsets, np.int64)
    s_in = dstruct(dev)
    rc = B.lib.bmxg_set_state(B.h, C.byref(s_in), off.ctypes.data_as(C.POINTER(C.c_int64)), BMXG_DEVICE)
    assert rc == 0, B.lib.bmxg_last_error(B.h)
    for ctx in (A, B):
        ctx.step(w.dt, 12, BMXG_FP32F)
        ctx.step(w.dt, 1, BMXG_FP64)
    QA = P.copy()
    A.get_state(QA, ("x", "y", "z", "velx", "vely", "velz"))
    s_out = dstruct(out)
    assert B.lib.bmxg_get_state(B.h, C.byref(s_out), BMXG_DEVICE) == 0
    torch.cuda.synchronize()
    for k, t in out.items():
        assert np.array_equal(t.cpu().numpy(), QA[k]), k


@pytest.mark.parametrize("precision", [BMXG_FP32F, BMXG_FP64])
def test_reloading_the_stored_state_keeps_the_trajectory(gpu_lib, precision):
    """A load-step-store loop that hands the stored positions back unchanged
    steps exactly as the device-resident loop: the load recognises the state
    bit for bit and keeps the neighbour list and its frames (FP32F), and the
    velocities it resets read as zero until the next step."""
    w = configs.colonies(ncol=8, nmin=2_000, nmax=20_000)
    fin = ("x", "y", "z", "radius", "cell_type")
    fout = ("x", "y", "z", "velx", "vely", "velz")
    A = w.particles.copy()
    ca = Context(w.params, w.geoms)
    ca.set_state(A, w.offsets)
    for _ in range(30):
        ca.step(w.dt, 1, precision)
    ca.get_state(A, fout)
    B = w.particles.copy()
    cb = Context(w.params, w.geoms)
    cb.set_state(B, w.offsets)
    for s in range(30):
        if s:
            cb.set_state(B, w.offsets, fields=fin)
            if s == 1:  # nothing stepped since the load: the velocities read as zero
                Z = B.copy()
                cb.get_state(Z, fout)
                assert not np.any(Z["velx"]) and not np.any(Z["vely"]) and not np.any(Z["velz"])
        cb.step(w.dt, 1, precision)
        cb.get_state(B, fout)
    for k in fout:
        assert np.array_equal(A[k], B[k]), k
    # one position a last bit off: a full load, the same as a fresh context's
    C1 = B.copy()
    C1["x"][7] = np.nextafter(C1["x"][7], 1.0)
    cb.set_state(C1, w.offsets, fields=fin)
    cb.step(w.dt, 1, precision)
    cb.get_state(C1, fout)
    D = B.copy()
    D["x"][7] = np.nextafter(D["x"][7], 1.0)
    cd = Context(w.params, w.geoms)
    cd.set_state(D, w.offsets, fields=fin)
    cd.step(w.dt, 1, precision)
    cd.get_state(D, fout)
    for k in fout:
        assert np.array_equal(C1[k], D[k]), k


def test_reload_reads_zero_velocities_after_either_form(gpu_lib):
    """A reload of the stored state resets the velocities whichever form
    stepped before it: after an FP64 step (its velocity planes written) and
    after FP32F steps (the FP64 planes left as the last load zeroed them)."""
    w = configs.colonies(ncol=4, nmin=2_000, nmax=8_000)
    fin = ("x", "y", "z", "radius", "cell_type")
    fout = ("x", "y", "z", "velx", "vely", "velz")
    B = w.particles.copy()
    cb = Context(w.params, w.geoms)
    cb.set_state(B, w.offsets, fields=fin)
    for form in (BMXG_FP64, BMXG_FP32F, BMXG_FP32F, BMXG_FP64, BMXG_FP64, BMXG_FP32F):
        cb.step(w.dt, 2, form)
        cb.get_state(B, fout)
        assert np.any(B["velz"])
        cb.set_state(B, w.offsets, fields=fin)
        Z = B.copy()
        cb.get_state(Z, fout)
        for k in ("velx", "vely", "velz"):
            assert not np.any(Z[k]), (form, k)
        for k in ("x", "y", "z"):
            assert np.array_equal(Z[k], B[k]), (form, k)
    cb.close()
