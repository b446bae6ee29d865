"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

liboracle.so is the plain-C restatement (bmx_oracle.c); _ref/libbmxref.so is
the reference's own force header and loop bodies compiled on the host
(ref_harness.cpp, only buildable where the reference tree is present).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from boltzmannmfx_gb300.abi import (BMXG_ERR_CAPACITY, BMXG_OK, Geometry, Params,
                                    Particles, ParticlesStruct, SplitParams)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libbmxref.so")
REF_TREE = os.environ.get("BMX_REFERENCE", "/root/reference")

_lib = None
_ref = None

_P = C.POINTER(Params)
_G = C.POINTER(Geometry)
_S = C.POINTER(ParticlesStruct)
_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_i64 = C.POINTER(C.c_int64)
_i8 = C.POINTER(C.c_int8)


def build(ref=None):
    """make the port (and the reference harness when the tree is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref is None:
        ref = os.path.isdir(os.path.join(REF_TREE, "src", "des"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        L = C.CDLL(LIB)
        L.orc_pairs.argtypes = [_P, _G, _S, _i64, _i32, _i8, C.c_int64, _i64]
        L.orc_forces.argtypes = [_P, _G, _S, _i64, _i32, _i8, _d, C.c_int]
        L.orc_update.argtypes = [_G, _S, _d, C.c_double, C.c_int]
        L.orc_update.restype = None
        L.orc_wrap.argtypes = [_G, _S]
        L.orc_wrap.restype = None
        L.orc_evolve.argtypes = [_P, C.c_int32, _G, _i64, _S, C.c_double, C.c_int32, C.c_int]
        L.orc_time_evolve.argtypes = [_P, C.c_int32, _G, _i64, _S, C.c_double, C.c_int32, C.c_int]
        L.orc_time_evolve.restype = C.c_double
        L.orc_pair_force.argtypes = [_P, _d, _S, C.c_int64, C.c_int64, _d, _d]
        L.orc_pair_force.restype = None
        L.orc_surface_force.argtypes = [_P, _S, C.c_int64, _d, _d]
        L.orc_surface_force.restype = None
        L.orc_min_distance.argtypes = [_d, _d, _d]
        L.orc_min_distance.restype = None
        L.orc_init_bonds.argtypes = [_P, _G, _S, _i64, _i32, _i8, C.c_double, _i64, _i64]
        L.orc_particle_exchange.argtypes = [_G, _S, _i64, _i32, _d, _d, C.c_double, _d]
        L.orc_split_cells_aos.argtypes = [C.POINTER(SplitParams), C.c_void_p, C.c_int64, C.c_int64, C.c_int32,
                                          C.c_int32, C.c_void_p, C.c_int64, C.c_uint64, C.c_int64, C.c_int32,
                                          _i64]
        L.orc_split_uniform.argtypes = [C.c_uint64, C.c_int32, C.c_int32, C.c_int32]
        L.orc_split_uniform.restype = C.c_double
        _lib = L
    return _lib


def have_ref():
    return os.path.exists(REFLIB)


def reflib():
    global _ref
    if _ref is None:
        if not os.path.exists(REFLIB):
            return None
        L = C.CDLL(REFLIB)
        L.ref_forces.argtypes = [_P, _G, _S, _i64, _i32, _i8, _d]
        L.ref_update.argtypes = [_G, _S, _d, C.c_double]
        L.ref_update.restype = None
        L.ref_min_distance.argtypes = [_d, _d, _d]
        L.ref_min_distance.restype = None
        L.ref_max_dist.argtypes = [_S, C.c_int64, C.c_int64, C.c_double]
        L.ref_max_dist.restype = C.c_double
        L.ref_pair_force.argtypes = [_P, _d, _S, C.c_int64, C.c_int64, _d, _d]
        L.ref_pair_force.restype = None
        L.ref_surface_force.argtypes = [_P, _S, C.c_int64, _d, _d]
        L.ref_surface_force.restype = None
        L.ref_init_bonds.argtypes = [_P, _G, _S, _i64, _i32, _i8, C.c_double]
        L.ref_particle_exchange.argtypes = [_S, _i64, _i32, _i8, _G, _d, _d, C.c_double, _d]
        L.ref_split_cells_aos.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.POINTER(SplitParams),
                                          C.c_void_p, C.c_int64, C.c_int64, C.c_int32, _i64, _i64]
        _ref = L
    return _ref


def _dp(a):
    return a.ctypes.data_as(_d)


def pairs(params, geom, P):
    """(offs int64[n+1], idx int32[], img int8[]) of the oracle's neighbour list."""
    L = lib()
    s = P.struct()
    offs = np.zeros(P.n + 1, np.int64)
    total = C.c_int64(0)
    rc = L.orc_pairs(C.byref(params), C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                     None, None, 0, C.byref(total))
    if rc not in (BMXG_OK, BMXG_ERR_CAPACITY):
        raise RuntimeError(f"orc_pairs failed: {rc}")
    cap = max(int(total.value), 1)
    idx = np.zeros(cap, np.int32)
    img = np.zeros(cap, np.int8)
    rc = L.orc_pairs(C.byref(params), C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                     idx.ctypes.data_as(_i32), img.ctypes.data_as(_i8), cap, C.byref(total))
    if rc != BMXG_OK:
        raise RuntimeError(f"orc_pairs failed: {rc}")
    return offs, idx[:total.value], img[:total.value]


def forces(params, geom, P, pl, nthreads=1, use_ref=False):
    """fc[6, n] of the force gather + wall force on list pl; mutates P's ints."""
    offs, idx, img = pl
    fc = np.zeros(6 * P.n, np.float64)
    s = P.struct()
    idx = np.ascontiguousarray(idx, np.int32)
    img = np.ascontiguousarray(img, np.int8)
    if len(idx) == 0:
        idx = np.zeros(1, np.int32)
        img = np.zeros(1, np.int8)
    if use_ref:
        L = reflib()
        rc = L.ref_forces(C.byref(params), C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                          idx.ctypes.data_as(_i32), img.ctypes.data_as(_i8), _dp(fc))
    else:
        rc = lib().orc_forces(C.byref(params), C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                              idx.ctypes.data_as(_i32), img.ctypes.data_as(_i8), _dp(fc), nthreads)
    if rc != BMXG_OK:
        raise RuntimeError(f"forces failed: {rc}")
    return fc.reshape(6, P.n)


def update(geom, P, fc, dt, use_ref=False, nthreads=1):
    fcf = np.ascontiguousarray(fc, np.float64).reshape(-1)
    s = P.struct()
    if use_ref:
        reflib().ref_update(C.byref(geom), C.byref(s), _dp(fcf), dt)
    else:
        lib().orc_update(C.byref(geom), C.byref(s), _dp(fcf), dt, nthreads)


def step(params, geom, P, dt, use_ref=False, nthreads=1):
    """One DEM step on a single colony; returns (pair list, fc)."""
    pl = pairs(params, geom, P)
    fc = forces(params, geom, P, pl, nthreads=nthreads, use_ref=use_ref)
    update(geom, P, fc, dt, use_ref=use_ref, nthreads=nthreads)
    return pl, fc


def _geoms_array(geoms):
    arr = (Geometry * len(geoms))()
    for k, g in enumerate(geoms):
        arr[k] = g
    return arr


def evolve(params, geoms, offsets, P, dt, nsteps, nthreads=1):
    arr = _geoms_array(geoms)
    off = np.ascontiguousarray(offsets, np.int64)
    s = P.struct()
    rc = lib().orc_evolve(C.byref(params), len(geoms), arr, off.ctypes.data_as(_i64),
                          C.byref(s), dt, nsteps, nthreads)
    if rc != BMXG_OK:
        raise RuntimeError(f"orc_evolve failed: {rc}")


def time_evolve(params, geoms, offsets, P, dt, nsteps, nthreads=1):
    arr = _geoms_array(geoms)
    off = np.ascontiguousarray(offsets, np.int64)
    s = P.struct()
    t = lib().orc_time_evolve(C.byref(params), len(geoms), arr, off.ctypes.data_as(_i64),
                              C.byref(s), dt, nsteps, nthreads)
    if t < 0:
        raise RuntimeError("orc_time_evolve failed")
    return t


def min_distance(e, use_ref=False):
    e = np.ascontiguousarray(e, np.float64)
    ti = C.c_double()
    tj = C.c_double()
    f = reflib().ref_min_distance if use_ref else lib().orc_min_distance
    f(_dp(e), C.byref(ti), C.byref(tj))
    return ti.value, tj.value


def pair_force(params, r12, P, i, j, use_ref=False):
    r = np.ascontiguousarray(r12, np.float64)
    v = np.zeros(3)
    w = np.zeros(3)
    f = reflib().ref_pair_force if use_ref else lib().orc_pair_force
    f(C.byref(params), _dp(r), C.byref(P.struct()), i, j, _dp(v), _dp(w))
    return v, w


def surface_force(params, P, i, use_ref=False):
    v = np.zeros(3)
    w = np.zeros(3)
    f = reflib().ref_surface_force if use_ref else lib().orc_surface_force
    f(C.byref(params), C.byref(P.struct()), i, _dp(v), _dp(w))
    return v, w


RLIM = 1.0e-7  # InitBonds' bond-detection distance (src/des/bmx_pc_interaction.cpp:508)


def init_bonds(params, geom, P, pl=None, rlim=RLIM, use_ref=False):
    """Bond segments whose ends are closer than rlim; mutates P's bond tables.
    Returns (added, overflow) for the port (None for the reference harness)."""
    offs, idx, img = pl if pl is not None else pairs(params, geom, P)
    idx = np.ascontiguousarray(idx if len(idx) else np.zeros(1, np.int32), np.int32)
    img = np.ascontiguousarray(img if len(img) else np.zeros(1, np.int8), np.int8)
    s = P.struct()
    if use_ref:
        # the reference's loop body and fixBonds printf per neighbour: send the
        # process's stdout to /dev/null around the call
        libc = C.CDLL(None)
        libc.fflush(None)
        saved = os.dup(1)
        null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(null, 1)
        try:
            rc = reflib().ref_init_bonds(C.byref(params), C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                                         idx.ctypes.data_as(_i32), img.ctypes.data_as(_i8), rlim)
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
            os.close(null)
        if rc != BMXG_OK:
            raise RuntimeError(f"ref_init_bonds failed: {rc}")
        return None
    added = C.c_int64(0)
    over = C.c_int64(0)
    rc = lib().orc_init_bonds(C.byref(params), C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                              idx.ctypes.data_as(_i32), img.ctypes.data_as(_i8), rlim, C.byref(added),
                              C.byref(over))
    if rc != BMXG_OK:
        raise RuntimeError(f"orc_init_bonds failed: {rc}")
    return added.value, over.value


def _quiet(call):
    """Run call() with the process's stdout sent to /dev/null (the
    reference's loop bodies print per particle)."""
    libc = C.CDLL(None)
    libc.fflush(None)
    saved = os.dup(1)
    null = os.open(os.devnull, os.O_WRONLY)
    os.dup2(null, 1)
    try:
        rc = call()
        libc.fflush(None)
    finally:
        os.dup2(saved, 1)
        os.close(saved)
        os.close(null)
    return rc


def particle_exchange(geom, P, vol, conc, dt, xpar, pl=None, params=None, use_ref=False):
    """One ParticleExchange substep; returns the new concentrations (3, n)."""
    if pl is None:
        pl = pairs(params, geom, P)
    offs, idx, img = pl
    idx = np.ascontiguousarray(idx if len(idx) else np.zeros(1, np.int32), np.int32)
    img = np.ascontiguousarray(img if len(img) else np.zeros(1, np.int8), np.int8)
    c = np.ascontiguousarray(conc, np.float64).reshape(-1).copy()
    v = np.ascontiguousarray(vol, np.float64)
    xp = np.ascontiguousarray(xpar, np.float64)
    s = P.struct()
    if use_ref:
        rc = _quiet(lambda: reflib().ref_particle_exchange(C.byref(s), offs.ctypes.data_as(_i64),
                                                           idx.ctypes.data_as(_i32), img.ctypes.data_as(_i8),
                                                           C.byref(geom), _dp(v), _dp(c), dt, _dp(xp)))
    else:
        rc = lib().orc_particle_exchange(C.byref(geom), C.byref(s), offs.ctypes.data_as(_i64),
                                         idx.ctypes.data_as(_i32), _dp(v), _dp(c), dt, _dp(xp))
    if rc != BMXG_OK:
        raise RuntimeError(f"particle exchange failed: {rc}")
    return c.reshape(3, P.n)


def split_cells(records, n, sp, draws=None, seed=0, next_id=1, my_proc=0, use_ref=False, return_used=False):
    """Cell division on AoS records (numpy, abi.aos_dtype(34, 35), room for the
    new particles), in place.  use_ref runs the reference's own split loop
    bodies (draw sequence only).  Returns (rc, number of new particles), and
    the draws the reference took when return_used."""
    out = C.c_int64(0)
    ptr = records.ctypes.data_as(C.c_void_p)
    if draws is not None:
        draws = np.ascontiguousarray(draws, dtype=np.float64)
    dptr = None if draws is None else draws.ctypes.data_as(C.c_void_p)
    nd = 0 if draws is None else draws.size
    if use_ref:
        used = C.c_int64(0)
        rc = _quiet(lambda: reflib().ref_split_cells_aos(ptr, int(n), len(records), C.byref(sp), dptr, nd,
                                                         int(next_id), int(my_proc), C.byref(out),
                                                         C.byref(used)))
        return (rc, out.value, used.value) if return_used else (rc, out.value)
    rc = lib().orc_split_cells_aos(C.byref(sp), ptr, int(n), len(records), 34, 35, dptr, nd,
                                   int(seed) & (2**64 - 1), int(next_id), int(my_proc), C.byref(out))
    return rc, out.value


def split_uniform(seed, ident, cpu, j):
    """Draw j of the seeded counter generator for the cell (ident, cpu)."""
    return lib().orc_split_uniform(int(seed) & (2**64 - 1), int(ident), int(cpu), int(j))

