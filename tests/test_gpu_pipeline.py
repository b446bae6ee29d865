"""The particle pipeline of bmx::Evolve (src/timestepping/bmx_evolve.cpp:95-99)
on the reference's own 410-segment hyphal network: EvolveParticles
(bmxg_evolve_particles_aos) then split_particles (bmxg_split_cells_aos), five
times over, on BMX's 448-byte particle records, against the oracle running
the same sequence (its FP64 step on the records' fields, its division on the
records).  The network grows by tip extension, two-way splits and side
branches between steps, so every step after the first runs on particles the
library itself appended.

Tolerance: integer fields (bond tables, positions on the hypha, ids) and the
division decisions exact; reals within 1e-9 of the field's scale (the FP64
rod step agrees within 1e-10 plus the reference's sensitivity to a last-bit
difference of sin/cos, and the divisions' acos/sin/cos add a few ulps)."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, runtime
from boltzmannmfx_gb300.abi import REAL_IDX as R, Particles, aos_dtype
from common import geom_of, load, params_of, particles_of, split_params
from test_gpu_aos import I as AI, NINT, NREAL, R as AR, to_aos

pytestmark = pytest.mark.gpu


def from_aos(a, n):
    """the step's fields of the first n records as particle arrays"""
    P = Particles(n, rods=True)
    P["x"], P["y"], P["z"] = a["pos"][:n, 0].copy(), a["pos"][:n, 1].copy(), a["pos"][:n, 2].copy()
    for k, j in AR.items():
        P[k] = a["rdata"][:n, j].copy()
    for k, j in AI.items():
        P[k] = a["idata"][:n, j].copy()
    P["seg_id1"] = a["idata"][:n, 7:11].T.reshape(-1).copy()
    P["seg_id2"] = a["idata"][:n, 11:15].T.reshape(-1).copy()
    P["site"] = a["idata"][:n, 15:19].T.reshape(-1).copy()
    P["dltd"] = a["idata"][:n, 26:32].T.reshape(-1).copy()
    return P


def into_aos(P, a):
    n = P.n
    b = to_aos(P)
    a["pos"][:n] = b["pos"]
    for j in list(AR.values()):
        a["rdata"][:n, j] = b["rdata"][:, j]
    for j in list(AI.values()) + list(range(7, 19)) + list(range(26, 32)):
        a["idata"][:n, j] = b["idata"][:, j]


def assert_close(g, r, n, what):
    for f in ("id", "cpu", "idata"):
        assert np.array_equal(g[f][:n], r[f][:n]), (what, f)
    gr, rr = g["rdata"][:n], r["rdata"][:n]
    scale = np.maximum(np.abs(rr).max(axis=0), 1e-300)
    err = (np.abs(gr - rr) / scale).max(axis=0)
    assert err.max() <= 1e-9, (what, int(err.argmax()), float(err.max()))
    perr = float(np.abs(g["pos"][:n] - r["pos"][:n]).max() / np.abs(r["pos"][:n]).max())
    assert perr <= 1e-9, (what, perr)


def test_evolve_then_split_on_the_hyphal_network(gpu_lib, oracle_lib):
    d = load("fungi_network")
    P0 = particles_of(d)
    prm, g = params_of(d), geom_of(d)
    dt = float(d["dt"])
    n = P0.n
    cap = 6 * n
    rec = np.zeros(cap, aos_dtype(NREAL, NINT))
    b = to_aos(P0)
    for f in ("pos", "rdata", "idata"):
        rec[f][:n] = b[f]
    rec["id"][:n], rec["cpu"][:n] = P0["id"], P0["cpu"]
    rec["rdata"][:n, R["vol"]] = np.pi * P0["radius"] ** 2 * P0["c_length"]
    ref = rec.copy()
    # tips at the radius limit split once they are at least 3.0e-3 long
    sp = split_params(max_len=0.0030, max_rad=0.00025, brnch_prob=0.3, split_prob=0.5, split_len=0.0025)
    ctx = Context(prm, [g])
    rng = np.random.default_rng(71)
    next_id = int(P0["id"].max()) + 1
    grown = 0
    for it in range(5):
        cost = (C.c_double * 1)()
        nsub = C.c_int32(0)
        rc = gpu_lib.bmxg_evolve_particles_aos(ctx.h, rec.ctypes.data_as(C.c_void_p), n, NREAL, NINT, None, dt,
                                               cost, C.byref(nsub))
        assert rc == 0, gpu_lib.bmxg_last_error(ctx.h)
        P = from_aos(ref, n)
        oracle_lib.step(prm, g, P, dt)
        into_aos(P, ref)
        assert_close(rec, ref, n, f"step {it}")
        draws = rng.random(8 * n)
        k = runtime.split_cells_aos(rec, n, sp, draws=draws, next_id=next_id, my_proc=0)
        rc, k2 = oracle_lib.split_cells(ref, n, sp, draws=draws, next_id=next_id, my_proc=0)
        assert rc == 0 and k == k2, (it, k, k2)
        n += k
        next_id += k
        grown += k
        assert_close(rec, ref, n, f"split {it}")
    assert grown > 0 and n <= cap
    # (id, cpu) names a particle: the checkpoint's came from 16 ranks, the new
    # ones from this call's rank 0 with ids past the largest
    key = rec["id"][:n].astype(np.int64) * 65536 + rec["cpu"][:n]
    assert len(np.unique(key)) == n
