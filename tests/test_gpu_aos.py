"""The reference-layout entry point: particles as amrex::Particle<34, 35>
structs (pos[3], rdata[34], id, cpu, idata[35]; 448 bytes) stepped through
bmxg_evolve_particles_aos, against the golden vectors of the reference's code."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300 import Context
from common import geom_of, load, params_of, particles_of, relerr, trig_floor, within

pytestmark = pytest.mark.gpu

NREAL, NINT = 34, 35
AOS = np.dtype([("pos", "<f8", 3), ("rdata", "<f8", NREAL), ("id", "<i4"), ("cpu", "<i4"),
                ("idata", "<i4", NINT), ("pad", "<i4", 1)])
R = dict(radius=0, c_length=1, theta=2, phi=3, area=4, velx=6, vely=7, velz=8, wx=9, wy=10, wz=11,
         bond_scale=24)
I = dict(cell_type=5, n_bnds=6, position=19, fuse_flag=20, split_flag=21, new_flag=22, fuse_tip=25,
         fix_site=32, id=33, cpu=34)


def to_aos(P):
    a = np.zeros(P.n, AOS)
    assert AOS.itemsize == 448
    a["pos"][:, 0], a["pos"][:, 1], a["pos"][:, 2] = P["x"], P["y"], P["z"]
    for k, j in R.items():
        a["rdata"][:, j] = P[k]
    for k, j in I.items():
        a["idata"][:, j] = P[k]
    n = P.n
    for k in range(4):
        a["idata"][:, 7 + k] = P["seg_id1"].reshape(4, n)[k]
        a["idata"][:, 11 + k] = P["seg_id2"].reshape(4, n)[k]
        a["idata"][:, 15 + k] = P["site"].reshape(4, n)[k]
    for k in range(6):
        a["idata"][:, 26 + k] = P["dltd"].reshape(6, n)[k]
    return a


@pytest.mark.parametrize("case", ["sphere_plain", "rods_small"])
def test_aos_entry_matches_golden(gpu_lib, oracle_lib, case):
    d = load(case)
    P = particles_of(d)
    fv, fw = trig_floor(oracle_lib, params_of(d), geom_of(d), P) if case != "sphere_plain" else (0.0, 0.0)
    ctx = Context(params_of(d), [geom_of(d)])
    a = to_aos(P)
    cost = (C.c_double * 1)()
    nsub = C.c_int32(0)
    rc = gpu_lib.bmxg_evolve_particles_aos(ctx.h, a.ctypes.data_as(C.c_void_p), P.n, NREAL, NINT, None,
                                           float(d["dt"]), cost, C.byref(nsub))
    assert rc == 0, gpu_lib.bmxg_last_error(ctx.h)
    assert nsub.value == 1 and cost[0] == P.n
    tol = 0.0 if case == "sphere_plain" else 1e-10
    for k, col in (("x", 0), ("y", 1), ("z", 2)):
        assert relerr(a["pos"][:, col], d["s1_" + k]) <= tol, k
    for k, floor in (("velx", fv), ("vely", fv), ("velz", fv), ("wx", fw), ("wy", fw), ("wz", fw)):
        ref = d["fc1"][["velx", "vely", "velz", "wx", "wy", "wz"].index(k)]
        scale = np.abs(d["fc1"][:3] if k.startswith("vel") else d["fc1"][3:]).max()
        assert np.abs(a["rdata"][:, R[k]] - ref).max() <= tol * scale + 8 * floor, k
    for k in ("theta", "phi"):
        assert relerr(a["rdata"][:, R[k]], d["s1_" + k]) <= tol, k
    for k in ("n_bnds", "position", "fix_site", "fuse_flag"):
        assert np.array_equal(a["idata"][:, I[k]], d["s1_" + k]), k
