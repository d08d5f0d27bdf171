"""ctypes mirror of include/ahfgpu.h.

The structures here are byte-for-byte the C ABI declared in
``include/ahfgpu.h``; ``tests/test_abi.py`` checks sizes and offsets against
the compiled library.  Everything above this module (the batch helpers, the
tests, bench.py) talks to the library only through these structs and the
exported ``ahfgpu_*`` functions.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

AHFGPU_OK = 0
AHFGPU_ERR_INVALID = -1
AHFGPU_ERR_OOM = -2
AHFGPU_ERR_CUDA = -3
AHFGPU_ERR_TIMEOUT = -4
AHFGPU_ERR_NO_DEVICE = -5
AHFGPU_ERR_CAPACITY = -6
AHFGPU_ERR_STATE = -7

PLAIN_FP64 = 0
BATCHED_FP64 = 1
BATCHED_FP32C = 2
MODES = {"plain_fp64": PLAIN_FP64, "batched_fp64": BATCHED_FP64, "batched_fp32c": BATCHED_FP32C}

HALO_EMPTY = 0x001
HALO_RAN_SORT = 0x002
HALO_RAN_RVIR0 = 0x004
HALO_RAN_UNBIND = 0x008
HALO_RAN_RVIR1 = 0x010
HALO_RAN_PROFILE = 0x020
HALO_NO_MBP = 0x040
HALO_REPLAYED = 0x100
HALO_NOBOUND = 0x200
HALO_STAGE_MASK = 0x07F | HALO_NOBOUND

PROF_FIELDS = [
    "r", "npart", "nvpart", "ovdens", "dens", "v2_circ", "v_esc2", "sig_v", "Ekin",
    "Epot", "Lx", "Ly", "Lz", "axis1", "E1x", "E1y", "E1z", "axis2", "E2x", "E2y",
    "E2z", "axis3", "E3x", "E3y", "E3z",
]
PROF_NFIELDS = len(PROF_FIELDS)


class Params(C.Structure):
    _fields_ = [
        ("VescTune", C.c_double),
        ("MINPART", C.c_int64),
        ("ovlim", C.c_double),
        ("rho_vir", C.c_double),
        ("r_fac", C.c_double),
        ("x_fac", C.c_double),
        ("v_fac", C.c_double),
        ("m_fac", C.c_double),
        ("rho_fac", C.c_double),
        ("phi_fac", C.c_double),
        ("Hubble", C.c_double),
    ]


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint64)


class Batch(C.Structure):
    _fields_ = [
        ("nhalo", C.c_int64),
        ("off", _up),
        ("x", _fp), ("y", _fp), ("z", _fp),
        ("vx", _fp), ("vy", _fp), ("vz", _fp),
        ("w", _fp),
        ("gidx", _up),
        ("cx", _dp), ("cy", _dp), ("cz", _dp),
    ]


class Particles(C.Structure):
    """ahfgpu_particles: a snapshot's particles (device pointers)."""
    _fields_ = [
        ("n", C.c_uint64),
        ("x", _fp), ("y", _fp), ("z", _fp),
        ("vx", _fp), ("vy", _fp), ("vz", _fp),
        ("w", _fp),
    ]


class Centres(C.Structure):
    """ahfgpu_centres: halo centres and gather radii (device pointers)."""
    _fields_ = [
        ("nhalo", C.c_int64),
        ("cx", _dp), ("cy", _dp), ("cz", _dp), ("rad", _dp),
    ]


class Halo(C.Structure):
    _fields_ = [
        ("npart", C.c_uint64),
        ("nbins", C.c_int32),
        ("flags", C.c_uint32),
        ("niter", C.c_int32),
        ("fix_rounds", C.c_int32),
        ("M_vir", C.c_double), ("R_vir", C.c_double), ("ovdens", C.c_double), ("Phi0", C.c_double),
        ("vel", C.c_double * 3),
        ("sigV", C.c_double), ("v_esc2", C.c_double), ("V2_max", C.c_double),
        ("R_max", C.c_double), ("r2", C.c_double),
        ("lambda_", C.c_double), ("lambdaE", C.c_double), ("Ekin", C.c_double),
        ("Epot", C.c_double), ("SurfP", C.c_double),
        ("pos_com", C.c_double * 3), ("com_offset", C.c_double),
        ("pos_mbp", C.c_double * 3), ("vel_mbp", C.c_double * 3), ("mbp_offset", C.c_double),
        ("AngMom", C.c_double * 3), ("axis", C.c_double * 3),
        ("E1", C.c_double * 3), ("E2", C.c_double * 3), ("E3", C.c_double * 3),
        ("fMhires", C.c_double), ("cNFW", C.c_double), ("R1", C.c_double), ("cR1", C.c_double),
    ]


# numpy view of Halo (same layout) so results become structured arrays
HALO_DTYPE = np.dtype({
    "names": [f[0] for f in Halo._fields_],
    "formats": [
        np.uint64, np.int32, np.uint32, np.int32, np.int32,
        *[np.float64] * 4, (np.float64, 3), *[np.float64] * 5, *[np.float64] * 5,
        (np.float64, 3), np.float64, (np.float64, 3), (np.float64, 3), np.float64,
        (np.float64, 3), (np.float64, 3), (np.float64, 3), (np.float64, 3), (np.float64, 3),
        *[np.float64] * 4,
    ],
    "offsets": [getattr(Halo, f[0]).offset for f in Halo._fields_],
    "itemsize": C.sizeof(Halo),
})


class Stats(C.Structure):
    _fields_ = [
        ("n_particles_in", C.c_uint64),
        ("n_kept", C.c_uint64),
        ("n_retest", C.c_uint64),
        ("n_replay_halos", C.c_uint64),
        ("n_key_ties", C.c_uint64),
        ("n_fp64_halos", C.c_uint64),
        ("n_launches", C.c_uint64),
        ("ms_device", C.c_double),
        ("ms_total", C.c_double),
        ("ms_plan", C.c_double),
        ("ms_h2d", C.c_double),
        ("ms_h2d_first", C.c_double),
        ("ms_pack", C.c_double),
        ("ms_d2h", C.c_double),
    ]


class Result(C.Structure):
    _fields_ = [
        ("nhalo", C.c_int64),
        ("halo", C.POINTER(Halo)),
        ("member_off", _up),
        ("member", _up),
        ("prof_off", _up),
        ("prof", _dp),
        ("stats", Stats),
        ("priv", C.c_void_p),
    ]


def _ptr(a, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


def make_batch(lists) -> tuple[Batch, list]:
    """Build a Batch from a HaloLists-like object (numpy arrays).

    Returns the struct and the list of arrays it points into (keep it alive).
    """
    keep = []

    def arr(a, dt):
        if a is None:
            return None
        b = np.ascontiguousarray(a, dtype=dt)
        keep.append(b)
        return b

    off = arr(lists.off, np.uint64)
    b = Batch()
    b.nhalo = len(off) - 1
    b.off = _ptr(off, C.c_uint64)
    for name in ("x", "y", "z", "vx", "vy", "vz"):
        setattr(b, name, _ptr(arr(getattr(lists, name), np.float32), C.c_float))
    b.w = _ptr(arr(lists.w, np.float32), C.c_float)
    b.gidx = _ptr(arr(lists.gidx, np.uint64), C.c_uint64)
    for name in ("cx", "cy", "cz"):
        setattr(b, name, _ptr(arr(getattr(lists, name), np.float64), C.c_double))
    return b, keep


class HostResult:
    """numpy copy of an ahfgpu_result (owned by Python)."""

    def __init__(self, r: Result):
        nh = int(r.nhalo)
        self.nhalo = nh
        if nh > 0:
            raw = np.ctypeslib.as_array(C.cast(r.halo, C.POINTER(C.c_uint8)), shape=(nh * C.sizeof(Halo),))
            self.halo = raw.view(HALO_DTYPE).copy()
        else:
            self.halo = np.zeros(0, dtype=HALO_DTYPE)
        self.member_off = np.ctypeslib.as_array(r.member_off, shape=(nh + 1,)).copy()
        nm = int(self.member_off[-1])
        self.member = (np.ctypeslib.as_array(r.member, shape=(nm,)).copy() if nm else np.zeros(0, np.uint64))
        self.prof_off = np.ctypeslib.as_array(r.prof_off, shape=(nh + 1,)).copy()
        nb = int(self.prof_off[-1])
        self.prof = (np.ctypeslib.as_array(r.prof, shape=(nb, PROF_NFIELDS)).copy() if nb
                     else np.zeros((0, PROF_NFIELDS)))
        s = r.stats
        self.stats = {f[0]: getattr(s, f[0]) for f in Stats._fields_}

    def members(self, h: int) -> np.ndarray:
        return self.member[self.member_off[h]:self.member_off[h + 1]]

    def profile(self, h: int) -> np.ndarray:
        return self.prof[self.prof_off[h]:self.prof_off[h + 1]]
