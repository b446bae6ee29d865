"""ctypes mirror of include/bmxg.h (structs, constants) and the particle container.

The C ABI takes plain pointers; this module only describes those structs for
Python callers (tests, bench.py, the torch wrapper of the adjoint) and owns
numpy arrays whose addresses are handed across the boundary.
"""
import ctypes as C

import numpy as np

BMXG_OK = 0
BMXG_ERR_ARG = -1
BMXG_ERR_CUDA = -2
BMXG_ERR_OOM = -3
BMXG_ERR_CAPACITY = -4
BMXG_ERR_STATE = -5
BMXG_ERR_NONFINITE = -6
BMXG_ERR_TIMEOUT = -7
BMXG_ERR_UNSUPPORTED = -8

BMXG_HOST = 0
BMXG_DEVICE = 1
BMXG_FP64 = 0
BMXG_FP32F = 1

YEAST = 0
FUNGI = 1
SITE_TIP, SITE_SECOND_1, SITE_SECOND_2, SITE_INTERIOR = 0, 1, 2, 3

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)


class Params(C.Structure):
    """bmxg_params: fpar[0..8] of BMXCellInteraction::getForceParams
    (src/chemistry/bmx_cell_interaction.cpp:84-93) + DEM::neighborhood."""
    _fields_ = [(n, C.c_double) for n in (
        "bndry_width", "stiffness", "z_wall", "z_bndry_width", "z_stiffness",
        "z_gravity", "bond_strength", "bond_cutoff", "viscosity", "neighborhood")]


class Geometry(C.Structure):
    _fields_ = [("prob_lo", C.c_double * 3), ("prob_hi", C.c_double * 3),
                ("n_cell", C.c_int32 * 3), ("is_periodic", C.c_int32 * 3)]

    @classmethod
    def make(cls, lo, hi, n_cell, periodic=(1, 1, 0)):
        g = cls()
        for d in range(3):
            g.prob_lo[d] = lo[d]
            g.prob_hi[d] = hi[d]
            g.n_cell[d] = int(n_cell[d])
            g.is_periodic[d] = int(periodic[d])
        return g

    def as_tuple(self):
        return (tuple(self.prob_lo), tuple(self.prob_hi), tuple(self.n_cell),
                tuple(self.is_periodic))


class ParticlesStruct(C.Structure):
    _fields_ = [("n", C.c_int64),
                ("x", _d), ("y", _d), ("z", _d),
                ("radius", _d), ("c_length", _d), ("theta", _d), ("phi", _d),
                ("area", _d), ("bond_scale", _d),
                ("velx", _d), ("vely", _d), ("velz", _d),
                ("wx", _d), ("wy", _d), ("wz", _d),
                ("cell_type", _i), ("id", _i), ("cpu", _i), ("n_bnds", _i),
                ("seg_id1", _i), ("seg_id2", _i), ("site", _i),
                ("position", _i), ("fuse_tip", _i), ("fix_site", _i),
                ("fuse_flag", _i), ("split_flag", _i), ("new_flag", _i),
                ("dltd", _i)]


class Stats(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("n_pairs_last", C.c_int64),
                ("n_out_of_domain", C.c_int64), ("n_edge_ghost", C.c_int64),
                ("n_bond_repairs", C.c_int64), ("n_rebins", C.c_int64),
                ("n_kernel_launches", C.c_int64), ("main_kernel_launches", C.c_int64),
                ("main_kernel_ms", C.c_double), ("last_step_ms", C.c_double)]


class Tile(C.Structure):
    """bmxg_tile: first and last cell per axis (0-based, inclusive)."""
    _fields_ = [("lo", C.c_int32 * 3), ("hi", C.c_int32 * 3)]


class Shapes(C.Structure):
    """bmxg_shapes: the launch shapes in use."""
    _fields_ = [("sphere_block", C.c_int32 * 2), ("sphere_grid", C.c_int32 * 2),
                ("list_step_block", C.c_int32), ("list_step_passes", C.c_int32),
                ("list_build_block", C.c_int32), ("list_step_persistent", C.c_int32)]


class SplitParams(C.Structure):
    """bmxg_split_params: parameters of the division step."""
    _fields_ = [("max_vol", C.c_double), ("overlap", C.c_double), ("max_len", C.c_double),
                ("max_rad", C.c_double), ("brnch_prob", C.c_double), ("split_prob", C.c_double),
                ("split_len", C.c_double), ("num_reals", C.c_int32), ("num_ints", C.c_int32)]


# positions in amrex::Particle's rdata / idata (realIdx, intIdx of
# src/chemistry/bmx_chem.H:38-118)
REAL_IDX = dict(radius=0, c_length=1, theta=2, phi=3, area=4, vol=5, velx=6, vely=7, velz=8,
                wx=9, wy=10, wz=11, fx=12, fy=13, fz=14, dadt=21, dvdt=22, tau_split=23,
                bond_scale=24, first_data=25)
INT_IDX = dict(cell_type=5, n_bnds=6, position=19, fuse_flag=20, split_flag=21, new_flag=22,
               fuse_tip=25, fix_site=32, id=33, cpu=34, first_data=35)


def aos_dtype(nreal=34, nint=35):
    """numpy dtype of amrex::Particle<nreal, nint> in AMReX 22.x, double
    precision: pos[3], rdata[nreal], id, cpu, idata[nint], padded to 8 bytes
    (448 bytes for BMX's 34 / 35)."""
    fields = [("pos", "<f8", 3), ("rdata", "<f8", nreal), ("id", "<i4"), ("cpu", "<i4"),
              ("idata", "<i4", nint)]
    if nint % 2:
        fields.append(("pad", "<i4"))
    return np.dtype(fields)


REAL_FIELDS = ("x", "y", "z", "radius", "c_length", "theta", "phi", "area",
               "bond_scale", "velx", "vely", "velz", "wx", "wy", "wz")
INT_FIELDS = ("cell_type", "id", "cpu", "n_bnds", "position", "fuse_tip",
              "fix_site", "fuse_flag", "split_flag", "new_flag")
PLANE_FIELDS = {"seg_id1": 4, "seg_id2": 4, "site": 4, "dltd": 6}


class Particles:
    """Host SoA particle state with the reference's field names.

    Arrays are numpy (float64 / int32).  `struct()` returns a ParticlesStruct
    pointing at them (the object keeps the arrays alive)."""

    def __init__(self, n, rods=False):
        self.n = int(n)
        self.a = {}
        for f in REAL_FIELDS:
            self.a[f] = np.zeros(self.n, np.float64)
        for f in INT_FIELDS:
            self.a[f] = np.zeros(self.n, np.int32)
        self.a["bond_scale"][:] = 1.0
        self.rods = rods
        for f, k in PLANE_FIELDS.items():
            self.a[f] = np.zeros(k * self.n, np.int32)
        self.a["dltd"][:] = -1
        self.a["id"][:] = np.arange(1, self.n + 1, dtype=np.int32)

    def __getitem__(self, k):
        return self.a[k]

    def __setitem__(self, k, v):
        self.a[k][...] = v

    def copy(self):
        q = Particles.__new__(Particles)
        q.n = self.n
        q.rods = self.rods
        q.a = {k: v.copy() for k, v in self.a.items()}
        return q

    def subset(self, lo, hi):
        """Particles lo..hi-1 as a new container (plane fields re-strided)."""
        q = Particles.__new__(Particles)
        q.n = hi - lo
        q.rods = self.rods
        q.a = {}
        for k, v in self.a.items():
            if k in PLANE_FIELDS:
                kk = PLANE_FIELDS[k]
                q.a[k] = v.reshape(kk, self.n)[:, lo:hi].copy().reshape(-1)
            else:
                q.a[k] = v[lo:hi].copy()
        return q

    @staticmethod
    def concat(parts):
        n = sum(p.n for p in parts)
        q = Particles.__new__(Particles)
        q.n = n
        q.rods = any(p.rods for p in parts)
        q.a = {}
        for k in parts[0].a:
            if k in PLANE_FIELDS:
                kk = PLANE_FIELDS[k]
                q.a[k] = np.concatenate([p.a[k].reshape(kk, p.n) for p in parts], axis=1).reshape(-1)
            else:
                q.a[k] = np.concatenate([p.a[k] for p in parts])
        return q

    def struct(self, fields=None):
        # the struct of the last call with the same fields, while it still
        # points at this container's arrays (a load-step-store loop builds it
        # once instead of every call)
        key = None if fields is None else tuple(fields)
        cache = self.__dict__.setdefault("_structs", {})
        hit = cache.get(key)
        if hit is not None and hit[0].n == self.n and all(self.a[k] is v for k, v in hit[1]):
            return hit[0]
        s = ParticlesStruct()
        s.n = self.n
        want = set(fields) if fields is not None else None
        used = []
        for name, ctype in ParticlesStruct._fields_[1:]:
            if want is not None and name not in want:
                setattr(s, name, ctype())
                continue
            arr = self.a[name]
            assert arr.flags["C_CONTIGUOUS"]
            setattr(s, name, arr.ctypes.data_as(ctype))
            used.append((name, arr))
        cache[key] = (s, tuple(used))
        return s

    def nbytes(self, fields):
        return sum(self.a[f].nbytes for f in fields)


SPHERE_IN_FIELDS = ("x", "y", "z", "radius", "cell_type")
SPHERE_OUT_FIELDS = ("x", "y", "z", "velx", "vely", "velz")
