"""Python binding of the C ABI in include/bmxg.h (ctypes; no torch types).

This is the host-side mirror of the reference's call for Python callers:
`Context.evolve_particles(dt)` is BMXParticleContainer::EvolveParticles
(src/des/bmx_pc.H:126-129) on the state loaded with `set_state`.  There is
no CPU fallback: constructing a Context without the built library or without
a CUDA device raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import Geometry, Params, Particles, ParticlesStruct, SplitParams, Stats

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbmxg.so")

_lib = None

# every entry point include/bmxg.h declares
ABI_SYMBOLS = ("bmxg_version", "bmxg_last_error", "bmxg_create", "bmxg_destroy", "bmxg_set_params",
               "bmxg_set_stream", "bmxg_set_state", "bmxg_get_state", "bmxg_step",
               "bmxg_evolve_particles", "bmxg_evolve_particles_aos", "bmxg_get_stats",
               "bmxg_set_profiling", "bmxg_get_pairs", "bmxg_set_ext", "bmxg_forward",
               "bmxg_backward", "bmxg_sphere_step_noalloc", "bmxg_init_bonds", "bmxg_set_list_mode",
               "bmxg_particle_exchange", "bmxg_read_ascii", "bmxg_write_ascii", "bmxg_write_vtk",
               "bmxg_read_checkpoint",
               "bmxg_io_last_error", "bmxg_autotune", "bmxg_get_shapes", "bmxg_step_tile", "bmxg_prepare", "bmxg_set_shapes", "bmxg_split_cells_aos", "bmxg_set_pair_capture",
               "bmxg_get_step_pairs")


class Ext(C.Structure):
    """bmxg_ext: extension parameters of the differentiation form."""
    _fields_ = [("damping", C.c_double), ("mu", C.c_double), ("adhesion", C.POINTER(C.c_double))]


class BmxgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"bmxg error {code}: {msg}")
        self.code = code


def load_library(path=None):
    """Load libbmxg.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with boltzmannmfx_gb300.build.build()")
    L = C.CDLL(p)
    vp = C.c_void_p
    L.bmxg_version.restype = C.c_int
    L.bmxg_last_error.restype = C.c_char_p
    L.bmxg_last_error.argtypes = [vp]
    L.bmxg_create.argtypes = [C.POINTER(Params), C.c_int32, C.POINTER(Geometry), C.POINTER(vp)]
    L.bmxg_destroy.argtypes = [vp]
    L.bmxg_destroy.restype = None
    L.bmxg_set_params.argtypes = [vp, C.POINTER(Params)]
    L.bmxg_set_stream.argtypes = [vp, vp]
    L.bmxg_set_state.argtypes = [vp, C.POINTER(ParticlesStruct), C.POINTER(C.c_int64), C.c_int]
    L.bmxg_get_state.argtypes = [vp, C.POINTER(ParticlesStruct), C.c_int]
    L.bmxg_step.argtypes = [vp, C.c_double, C.c_int32, C.c_int32]
    L.bmxg_prepare.argtypes = [vp, C.c_double, C.c_int32]
    L.bmxg_step_tile.argtypes = [vp, C.POINTER(abi.Tile), C.POINTER(ParticlesStruct), C.POINTER(ParticlesStruct),
                                 C.c_double, C.c_int32]
    L.bmxg_evolve_particles.argtypes = [vp, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    L.bmxg_evolve_particles_aos.argtypes = [vp, vp, C.c_int64, C.c_int32, C.c_int32,
                                            C.POINTER(C.c_int64), C.c_double, C.POINTER(C.c_double),
                                            C.POINTER(C.c_int32)]
    L.bmxg_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.bmxg_set_profiling.argtypes = [vp, C.c_int32]
    L.bmxg_get_pairs.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int8),
                                 C.c_int64, C.POINTER(C.c_int64)]
    L.bmxg_autotune.argtypes = [vp, C.c_char_p]
    L.bmxg_get_shapes.argtypes = [vp, C.POINTER(abi.Shapes)]
    L.bmxg_set_shapes.argtypes = [vp, C.POINTER(abi.Shapes)]
    L.bmxg_init_bonds.argtypes = [vp, C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.bmxg_set_list_mode.argtypes = [vp, C.c_int32]
    L.bmxg_set_pair_capture.argtypes = [vp, C.c_int32]
    L.bmxg_get_step_pairs.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int64,
                                      C.POINTER(C.c_int64)]
    dp = C.POINTER(C.c_double)
    L.bmxg_particle_exchange.argtypes = [vp, dp, dp, C.c_double, dp, C.c_int32]
    PS = C.POINTER(ParticlesStruct)
    L.bmxg_read_ascii.argtypes = [C.c_char_p, PS, C.c_int64, C.POINTER(C.c_int64)]
    L.bmxg_write_ascii.argtypes = [C.c_char_p, PS]
    L.bmxg_write_vtk.argtypes = [C.c_char_p, PS, C.POINTER(C.c_double)]
    L.bmxg_read_checkpoint.argtypes = [C.c_char_p, C.c_int32, PS, C.c_int64, C.POINTER(C.c_int64)]
    L.bmxg_io_last_error.restype = C.c_char_p
    L.bmxg_io_last_error.argtypes = []
    L.bmxg_set_ext.argtypes = [vp, C.POINTER(Ext)]
    L.bmxg_sphere_step_noalloc.argtypes = [C.POINTER(Params), C.POINTER(Geometry), C.c_int64] + [vp] * 10 + \
        [C.c_double, vp, C.POINTER(C.c_int64)]
    L.bmxg_split_cells_aos.argtypes = [C.POINTER(SplitParams), vp, C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                       vp, C.c_int64, C.c_uint64, C.c_int64, C.c_int32, C.c_int32,
                                       C.POINTER(C.c_int64), vp]
    L.bmxg_forward.argtypes = [vp, C.c_double, C.c_int32, C.c_int32]
    L.bmxg_backward.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_double)]
    if path is None:
        _lib = L
    return L


def _geoms_array(geoms):
    arr = (Geometry * len(geoms))()
    for k, g in enumerate(geoms):
        arr[k] = g
    return arr


class Context:
    """One DEM state on the current CUDA device (one host thread at a time)."""

    def __init__(self, params, geoms):
        self.lib = load_library()
        if isinstance(geoms, Geometry):
            geoms = [geoms]
        self.params = params
        self.geoms = list(geoms)
        self._garr = _geoms_array(self.geoms)
        h = C.c_void_p()
        rc = self.lib.bmxg_create(C.byref(params), len(self.geoms), self._garr, C.byref(h))
        if rc != abi.BMXG_OK:
            raise BmxgError(rc, "bmxg_create failed (is a CUDA device visible?)")
        self.h = h
        self.n = 0

    def _check(self, rc):
        if rc != abi.BMXG_OK:
            raise BmxgError(rc, self.lib.bmxg_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.bmxg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self.params = params
        self._check(self.lib.bmxg_set_params(self.h, C.byref(params)))

    def set_stream(self, handle):
        self._check(self.lib.bmxg_set_stream(self.h, C.c_void_p(handle)))

    def set_state(self, P, offsets=None, where=abi.BMXG_HOST, fields=None):
        s = P.struct(fields)
        off = None
        if offsets is not None and len(self.geoms) > 1:
            # (the same offsets array as the last call: its int64 copy and pointer are kept)
            if getattr(self, "_off_src", None) is not offsets or not np.array_equal(self._off, offsets):
                self._off = np.array(offsets, np.int64)
                self._off_ptr = self._off.ctypes.data_as(C.POINTER(C.c_int64))
                self._off_src = offsets
            off = self._off_ptr
        self._check(self.lib.bmxg_set_state(self.h, C.byref(s), off, where))
        self.n = P.n

    def step(self, dt, nsteps=1, precision=abi.BMXG_FP64):
        self._check(self.lib.bmxg_step(self.h, dt, nsteps, precision))

    def prepare(self, dt, precision=abi.BMXG_FP64):
        """Instantiate the step graphs of (dt, precision) without stepping (bmxg_prepare)."""
        self._check(self.lib.bmxg_prepare(self.h, dt, precision))

    def step_tile(self, lo, hi, reals, ghosts, dt):
        """One FP64 step of the spheres of tile [lo, hi] (cells, inclusive) with
        the caller's ghosts (bmxg_step_tile): reals' x, y, z and velx, vely,
        velz are written in place."""
        t = abi.Tile()
        t.lo[:] = [int(v) for v in lo]
        t.hi[:] = [int(v) for v in hi]
        sr = reals.struct(("x", "y", "z", "radius", "cell_type", "velx", "vely", "velz"))
        sg = ghosts.struct(("x", "y", "z", "radius", "cell_type")) if ghosts is not None and ghosts.n else None
        self._check(self.lib.bmxg_step_tile(self.h, C.byref(t), C.byref(sr), C.byref(sg) if sg else None, dt,
                                            abi.BMXG_HOST))
        return reals

    def evolve_particles(self, dt):
        cost = (C.c_double * len(self.geoms))()
        nsub = C.c_int32(0)
        self._check(self.lib.bmxg_evolve_particles(self.h, dt, cost, C.byref(nsub)))
        return list(cost), nsub.value

    def get_state(self, P, fields=None, where=abi.BMXG_HOST):
        s = P.struct(fields)
        self._check(self.lib.bmxg_get_state(self.h, C.byref(s), where))
        return P

    def stats(self):
        st = Stats()
        self._check(self.lib.bmxg_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in Stats._fields_}

    def set_profiling(self, on):
        self._check(self.lib.bmxg_set_profiling(self.h, 1 if on else 0))

    def pairs(self):
        offs = np.zeros(self.n + 1, np.int64)
        total = C.c_int64(0)
        rc = self.lib.bmxg_get_pairs(self.h, offs.ctypes.data_as(C.POINTER(C.c_int64)), None, None, 0,
                                     C.byref(total))
        if rc not in (abi.BMXG_OK, abi.BMXG_ERR_CAPACITY):
            self._check(rc)
        cap = max(int(total.value), 1)
        idx = np.zeros(cap, np.int32)
        img = np.zeros(cap, np.int8)
        self._check(self.lib.bmxg_get_pairs(self.h, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                            idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                            img.ctypes.data_as(C.POINTER(C.c_int8)), cap, C.byref(total)))
        return offs, idx[:total.value], img[:total.value]

    def particle_exchange(self, vol, conc, dt, xpar):
        """One ParticleExchange substep on the loaded state: returns the new
        concentrations (3, n) of species A, B, C (caller order)."""
        c = np.ascontiguousarray(conc, np.float64).reshape(-1).copy()
        v = np.ascontiguousarray(vol, np.float64)
        x = np.ascontiguousarray(xpar, np.float64)
        dp = C.POINTER(C.c_double)
        self._check(self.lib.bmxg_particle_exchange(self.h, v.ctypes.data_as(dp), c.ctypes.data_as(dp), dt,
                                                    x.ctypes.data_as(dp), abi.BMXG_HOST))
        return c.reshape(3, self.n)

    def set_list_mode(self, mode):
        """1: FP32F sphere steps use the skin neighbour list where it is exact; 0: never."""
        self._check(self.lib.bmxg_set_list_mode(self.h, int(mode)))

    def set_pair_capture(self, on):
        """list steps record the pairs that pass the force gate (debug export)."""
        self._check(self.lib.bmxg_set_pair_capture(self.h, 1 if on else 0))

    def step_pairs(self):
        """(offs, idx): the gated pairs the last FP32F list step accumulated, per
        particle in original order, neighbours as original indices in the order
        the step summed them (needs set_pair_capture(True) before the step)."""
        offs = np.zeros(self.n + 1, np.int64)
        total = C.c_int64(0)
        rc = self.lib.bmxg_get_step_pairs(self.h, offs.ctypes.data_as(C.POINTER(C.c_int64)), None, 0,
                                          C.byref(total))
        if rc not in (abi.BMXG_OK, abi.BMXG_ERR_CAPACITY) or (rc == abi.BMXG_ERR_CAPACITY and total.value == 0):
            self._check(rc)
        idx = np.zeros(max(total.value, 1), np.int32)
        self._check(self.lib.bmxg_get_step_pairs(self.h, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                                 idx.ctypes.data_as(C.POINTER(C.c_int32)), total.value,
                                                 C.byref(total)))
        return offs, idx[:total.value]

    def init_bonds(self, rlim=1.0e-7):
        """InitBonds on the loaded state (bond tables of coincident segment
        ends).  Returns (added, overflow); raises BmxgError when a table is full."""
        added = C.c_int64(0)
        over = C.c_int64(0)
        rc = self.lib.bmxg_init_bonds(self.h, rlim, C.byref(added), C.byref(over))
        if rc == abi.BMXG_ERR_CAPACITY:
            raise BmxgError(rc, f"InitBonds: {over.value} bonds found a full table ({added.value} added)")
        self._check(rc)
        return added.value, over.value

    def set_ext(self, damping=0.0, mu=0.0, adhesion=None):
        e = Ext()
        e.damping = damping
        e.mu = mu
        self._adh = None if adhesion is None else np.ascontiguousarray(adhesion, np.float64)
        e.adhesion = (self._adh.ctypes.data_as(C.POINTER(C.c_double)) if self._adh is not None
                      else C.POINTER(C.c_double)())
        self._check(self.lib.bmxg_set_ext(self.h, C.byref(e)))

    def forward(self, dt, nsteps, ckpt_every=20):
        self._check(self.lib.bmxg_forward(self.h, dt, nsteps, ckpt_every))

    def backward(self, dL_dx):
        """dL_dx: (3, n) gradient w.r.t. the final positions.  Returns
        (dL/dx0 (3, n), dL/d(stiffness, damping, mu) (3,), dL/dadhesion (n,))."""
        g = np.ascontiguousarray(dL_dx, np.float64).reshape(-1)
        gx0 = np.zeros(3 * self.n)
        gp = np.zeros(3)
        ga = np.zeros(self.n)
        dp = C.POINTER(C.c_double)
        self._check(self.lib.bmxg_backward(self.h, g.ctypes.data_as(dp), gx0.ctypes.data_as(dp),
                                           gp.ctypes.data_as(dp), ga.ctypes.data_as(dp)))
        return gx0.reshape(3, self.n), gp, ga

    def autotune(self, cache_path=None):
        self._check(self.lib.bmxg_autotune(self.h, cache_path.encode() if cache_path else None))

    def set_shapes(self, **kw):
        """Pin launch shapes (bmxg_set_shapes): the current ones with the given keys replaced."""
        cur = self.shapes()
        cur.update(kw)
        sh = abi.Shapes()
        sh.sphere_block[:] = cur["sphere_block"]
        sh.sphere_grid[:] = cur["sphere_grid"]
        sh.list_step_block = cur["list_step_block"]
        sh.list_step_passes = cur["list_step_passes"]
        sh.list_build_block = cur["list_build_block"]
        sh.list_step_persistent = 1 if cur["list_step_persistent"] else 0
        self._check(self.lib.bmxg_set_shapes(self.h, C.byref(sh)))

    def shapes(self):
        """The launch shapes in use (bmxg_get_shapes)."""
        sh = abi.Shapes()
        self._check(self.lib.bmxg_get_shapes(self.h, C.byref(sh)))
        return {"sphere_block": list(sh.sphere_block), "sphere_grid": list(sh.sphere_grid),
                "list_step_block": sh.list_step_block, "list_step_passes": sh.list_step_passes,
                "list_build_block": sh.list_build_block, "list_step_persistent": bool(sh.list_step_persistent)}


# ---- fixture I/O (host functions of libbmxg.so; no device needed) -------------

def _io_check(L, rc):
    if rc != abi.BMXG_OK:
        raise BmxgError(rc, L.bmxg_io_last_error().decode())


def _two_call(read, *args):
    """Count with a NULL buffer, then fill a Particles of that size."""
    L = load_library()
    n = C.c_int64(0)
    rc = read(*args, None, 0, C.byref(n))
    if rc not in (abi.BMXG_OK, abi.BMXG_ERR_CAPACITY):
        _io_check(L, rc)
    P = Particles(n.value, rods=True)
    s = P.struct()
    _io_check(L, read(*args, C.byref(s), n.value, C.byref(n)))
    P.rods = bool((P["cell_type"] == abi.FUNGI).any())
    return P


def read_ascii(path):
    """Particles of a particle input file of the reference
    (BMXParticleContainer::InitParticlesAscii format)."""
    L = load_library()
    return _two_call(L.bmxg_read_ascii, os.fsencode(path))


def write_ascii(path, P):
    L = load_library()
    _io_check(L, L.bmxg_write_ascii(os.fsencode(path), C.byref(P.struct())))


def write_vtk(path, P, conc_b=None):
    """Legacy-VTK polydata as BMXParticleContainer::WriteToAscii writes it."""
    L = load_library()
    c = None if conc_b is None else np.ascontiguousarray(conc_b, np.float64)
    cp = c.ctypes.data_as(C.POINTER(C.c_double)) if c is not None else None
    _io_check(L, L.bmxg_write_vtk(os.fsencode(path), C.byref(P.struct()), cp))


def read_checkpoint(particles_dir, level=-1):
    """Particles of an AMReX checkpoint (Version_Two_Dot_One_double);
    particles_dir is the checkpoint's `particles` directory."""
    L = load_library()
    return _two_call(L.bmxg_read_checkpoint, os.fsencode(particles_dir), int(level))


def split_cells_aos(records, n, sp, draws=None, seed=0, next_id=1, my_proc=0, where=abi.BMXG_HOST,
                    nreal=34, nint=35, cap=None, stream=None):
    """Cell division (bmxg_split_cells_aos) on AoS records.

    where=BMXG_HOST: `records` is a numpy array of abi.aos_dtype(nreal, nint)
    holding n particles and room for the new ones (len(records) = cap), and
    `draws` a float64 numpy array (the draw sequence) or None (the seeded
    counter generator).  where=BMXG_DEVICE: `records` is a device address
    (an int, e.g. tensor.data_ptr()), `draws` None or (device address, count),
    and `cap` is required.  Returns the number of new particles; raises
    BmxgError."""
    L = load_library()
    if where == abi.BMXG_HOST:
        if records.dtype != abi.aos_dtype(nreal, nint):
            raise ValueError("records must have abi.aos_dtype(nreal, nint)")
        cap = len(records) if cap is None else cap
        ptr = records.ctypes.data_as(C.c_void_p)
        if draws is not None:
            draws = np.ascontiguousarray(draws, dtype=np.float64)
            nd, dptr = draws.size, draws.ctypes.data_as(C.c_void_p)
        else:
            nd, dptr = 0, None
    else:
        if cap is None:
            raise ValueError("cap is required for device records")
        ptr = C.c_void_p(int(records))
        nd, dptr = (0, None) if draws is None else (int(draws[1]), C.c_void_p(int(draws[0])))
    out = C.c_int64(0)
    rc = L.bmxg_split_cells_aos(C.byref(sp), ptr, int(n), int(cap), int(nreal), int(nint), dptr, int(nd),
                                int(seed) & (2**64 - 1), int(next_id), int(my_proc), int(where), C.byref(out),
                                None if stream is None else C.c_void_p(int(stream)))
    if rc != abi.BMXG_OK:
        raise BmxgError(rc, f"split_cells_aos ({out.value} divisions)")
    return out.value
