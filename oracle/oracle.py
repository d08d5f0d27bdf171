"""Python loader for the parity oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU
baseline leg import this module.  It loads

  oracle/_build/libahforacle.so   the C restatement (ahf_oracle.c), and
  oracle/_ref/libahfref[_mm].so   the reference's own routines driven by
                                  ref_harness.c (only where they were built;
                                  libahfref_bin.so: the -DAHFbinary build)

and returns ahf_gb300.abi.HostResult objects, the same shape the GPU library
returns.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

from ahf_gb300.abi import HostResult, Params, Result, make_batch

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict = {}


REPO = os.path.dirname(HERE)
# The reference's sources as a build input for machines without the AHF tree:
# a git-ignored mirror of its src/ directory, refreshed whenever the tree is
# present.  Nothing of it is committed; it only lets the same recipe compile
# the reference's own routines where the tree itself is absent.
REF_MIRROR = os.path.join(REPO, "baseline", "_ref")


def _mirror_reference(refdir: str) -> None:
    import shutil
    src = os.path.join(refdir, "src")
    dst = os.path.join(REF_MIRROR, "src")
    for root, _dirs, files in os.walk(src):
        rel = os.path.relpath(root, src)
        os.makedirs(os.path.join(dst, rel), exist_ok=True)
        for f in files:
            if not f.endswith((".c", ".h")):
                continue
            a, b = os.path.join(root, f), os.path.join(dst, rel, f)
            if not os.path.exists(b) or os.path.getmtime(b) < os.path.getmtime(a):
                shutil.copy2(a, b)


def reference_tree() -> str | None:
    """The AHF source tree to compile the reference from: $AHF_REFERENCE, the
    reference checkout, or the git-ignored mirror of it (refreshed from the
    checkout when that is present)."""
    env = os.environ.get("AHF_REFERENCE")
    if env:
        return env if os.path.isfile(os.path.join(env, "src/libahf/ahf_halos.c")) else None
    if os.path.isfile("/root/reference/src/libahf/ahf_halos.c"):
        _mirror_reference("/root/reference")
    if os.path.isfile(os.path.join(REF_MIRROR, "src/libahf/ahf_halos.c")):
        return REF_MIRROR
    return None


def build(ref: bool | None = None) -> None:
    """Compile the restatement (and the reference harness when the reference
    tree, or its mirror, is present and `ref` is not False)."""
    targets = ["oracle"]
    refdir = reference_tree() if ref is not False else None
    if refdir:
        targets.append("ref")
    jobs = str(min(8, os.cpu_count() or 1))
    subprocess.run(["make", "-s", "-j", jobs, "-C", HERE, f"REF={refdir or '/nonexistent'}", *targets], check=True)


def build_ahf() -> tuple[str, str]:
    """The whole AHF program from the reference tree (or its mirror): the
    stock serial build and the build with the stage swapped for the GPU
    library (oracle/Makefile target `ahf`).  Returns their paths."""
    refdir = reference_tree()
    if not refdir:
        raise FileNotFoundError("no AHF source tree (reference checkout or its mirror)")
    jobs = str(min(16, os.cpu_count() or 1))
    subprocess.run(["make", "-s", "-j", jobs, "-C", HERE, f"REF={refdir}", "ahf"], check=True)
    return os.path.join(HERE, "_ref", "ahf", "AHF"), os.path.join(HERE, "_ref", "ahf", "AHF-gpu")


def _load(path: str, prefix: str):
    if path in _LIBS:
        return _LIBS[path]
    lib = C.CDLL(path)
    fn = getattr(lib, f"{prefix}_construct_halos")
    fn.argtypes = [C.POINTER(Params), C.c_void_p, C.POINTER(Result), C.c_int]
    fn.restype = C.c_int
    fr = getattr(lib, f"{prefix}_result_free")
    fr.argtypes = [C.POINTER(Result)]
    fr.restype = None
    _LIBS[path] = (lib, fn, fr)
    return _LIBS[path]


def oracle_path() -> str:
    return os.path.join(HERE, "_build", "libahforacle.so")


def ref_path(multimass: bool) -> str:
    return os.path.join(HERE, "_ref", "libahfref_mm.so" if multimass else "libahfref.so")


def ref_bin_path() -> str:
    return os.path.join(HERE, "_ref", "libahfref_bin.so")


def have_ref(multimass: bool = False) -> bool:
    return os.path.isfile(ref_path(multimass))


def _run(path, prefix, params, lists, nthreads):
    lib, fn, fr = _load(path, prefix)
    b, keep = make_batch(lists)
    r = Result()
    rc = fn(C.byref(params), C.cast(C.pointer(b), C.c_void_p), C.byref(r), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"{prefix}_construct_halos failed: {rc}")
    try:
        return HostResult(r)
    finally:
        fr(C.byref(r))
        del keep


def run_oracle(params, lists, nthreads: int = 1) -> HostResult:
    """The C restatement, `nthreads` OpenMP threads (<=0: all)."""
    if not os.path.isfile(oracle_path()):
        build(ref=False)
    return _run(oracle_path(), "ahforacle", params, lists, nthreads)


def run_reference(params, lists, nthreads: int = 1) -> HostResult:
    """The reference's own routines (needs oracle/_ref built here)."""
    mm = lists.w is not None
    if not have_ref(mm):
        raise FileNotFoundError(ref_path(mm))
    return _run(ref_path(mm), "ahfref", params, lists, nthreads)


def max_threads() -> int:
    lib, _, _ = _load(oracle_path(), "ahforacle")
    lib.ahforacle_max_threads.restype = C.c_int
    return int(lib.ahforacle_max_threads())


def _gather(path: str, prefix: str, x, y, z, cx, cy, cz, rad):
    import numpy as np
    lib = C.CDLL(path)
    fn = getattr(lib, f"{prefix}_gather")
    fn.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.POINTER(C.c_uint64))]
    fn.restype = C.c_int
    fr = getattr(lib, f"{prefix}_gather_free")
    fr.argtypes = [C.POINTER(C.c_uint64)]
    fr.restype = None
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
    cen = [np.ascontiguousarray(a, dtype=np.float64) for a in (cx, cy, cz, rad)]
    nh = len(cen[0])
    off = np.zeros(nh + 1, np.uint64)
    pidx = C.POINTER(C.c_uint64)()
    rc = fn(len(arrs[0]), *[a.ctypes.data for a in arrs], nh, *[a.ctypes.data for a in cen], off.ctypes.data,
            C.byref(pidx))
    if rc != 0:
        raise RuntimeError(f"{prefix}_gather failed ({rc})")
    tot = int(off[-1])
    idx = np.ctypeslib.as_array(pidx, shape=(max(tot, 1),))[:tot].copy() if tot else np.zeros(0, np.uint64)
    fr(pidx)
    return off, idx


def gather_oracle(x, y, z, cx, cy, cz, rad):
    """CSR (off, idx) of the restated gather: every particle within each
    halo's radius, ascending index."""
    return _gather(oracle_path(), "ahforacle", x, y, z, cx, cy, cz, rad)


def gather_reference(x, y, z, cx, cy, cz, rad):
    """CSR (off, idx) of the reference's own SFC gather (its order)."""
    return _gather(ref_path(False), "ahfref", x, y, z, cx, cy, cz, rad)


def gather_radii_oracle(npart, cx, cy, cz, rvir, max_gather_rad_box: float):
    """The restated gather-radius loop (spatialRef2halos)."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_gather_radii
    fn.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    fn.restype = None
    a = [np.ascontiguousarray(npart, dtype=np.uint64)] + [np.ascontiguousarray(v, dtype=np.float64)
                                                          for v in (cx, cy, cz, rvir)]
    out = np.zeros(len(a[0]))
    fn(len(a[0]), *[v.ctypes.data for v in a], float(max_gather_rad_box), out.ctypes.data)
    return out


def _writer(path: str, prefix: str, ids, w, member_off, member, halo_npart, order, minpart: int, ref: bool):
    import tempfile
    import numpy as np
    lib = C.CDLL(path)
    fr = getattr(lib, f"{prefix}_write_free" if ref else "ahforacle_gather_free")
    a = dict(ids=np.ascontiguousarray(ids, dtype=np.uint64), off=np.ascontiguousarray(member_off, dtype=np.uint64),
             mem=np.ascontiguousarray(member, dtype=np.uint64), np_=np.ascontiguousarray(halo_npart, dtype=np.uint64),
             order=np.ascontiguousarray(order, dtype=np.int64))
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
    out = C.POINTER(C.c_ubyte)()
    nb = C.c_uint64()
    nh = len(a["np_"])
    if ref:
        fn = getattr(lib, f"{prefix}_write_particles")
        fn.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                       C.c_int64, C.c_char_p, C.POINTER(C.POINTER(C.c_ubyte)), C.POINTER(C.c_uint64)]
        fn.restype = C.c_int
        with tempfile.TemporaryDirectory() as d:
            rc = fn(len(a["ids"]), a["ids"].ctypes.data, wa.ctypes.data if wa is not None else None, nh,
                    a["off"].ctypes.data, a["mem"].ctypes.data, a["np_"].ctypes.data, a["order"].ctypes.data,
                    int(minpart), os.path.join(d, "ref").encode(), C.byref(out), C.byref(nb))
    else:
        fn = lib.ahforacle_write_particles
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                       C.POINTER(C.POINTER(C.c_ubyte)), C.POINTER(C.c_uint64)]
        fn.restype = C.c_int
        rc = fn(a["ids"].ctypes.data, wa.ctypes.data if wa is not None else None, nh, a["off"].ctypes.data,
                a["mem"].ctypes.data, a["np_"].ctypes.data, a["order"].ctypes.data, int(minpart), C.byref(out),
                C.byref(nb))
    if rc != 0:
        raise RuntimeError(f"writer failed ({rc})")
    data = bytes(np.ctypeslib.as_array(out, shape=(max(nb.value, 1),))[:nb.value])
    if ref:
        fr.argtypes = [C.c_void_p]
        fr(C.cast(out, C.c_void_p))
    else:
        C.CDLL(None).free.argtypes = [C.c_void_p]
        C.CDLL(None).free(C.cast(out, C.c_void_p))
    return data


def write_particles_oracle(ids, w, member_off, member, halo_npart, order, minpart: int) -> bytes:
    """The restated AHF_particles bytes."""
    return _writer(oracle_path(), "ahforacle", ids, w, member_off, member, halo_npart, order, minpart, False)


def write_particles_reference(ids, w, member_off, member, halo_npart, order, minpart: int) -> bytes:
    """The reference's own writer (ahf_io_WriteParticles), file read back."""
    return _writer(ref_path(w is not None), "ahfref", ids, w, member_off, member, halo_npart, order, minpart, True)


def write_particles_bin_oracle(ids, member_off, member, halo_npart, order, minpart: int) -> bytes:
    """The restated AHF_particles_bin bytes (ahf_binwrite_particles)."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_write_particles_bin
    fn.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                   C.POINTER(C.POINTER(C.c_ubyte)), C.POINTER(C.c_uint64)]
    fn.restype = C.c_int
    a = [np.ascontiguousarray(v, dtype=np.uint64) for v in (ids, member_off, member, halo_npart)]
    o = np.ascontiguousarray(order, dtype=np.int64)
    out = C.POINTER(C.c_ubyte)()
    nb = C.c_uint64()
    if fn(a[0].ctypes.data, len(a[3]), a[1].ctypes.data, a[2].ctypes.data, a[3].ctypes.data, o.ctypes.data,
          int(minpart), C.byref(out), C.byref(nb)) != 0:
        raise RuntimeError("binary writer failed")
    data = bytes(np.ctypeslib.as_array(out, shape=(max(nb.value, 1),))[:nb.value])
    C.CDLL(None).free.argtypes = [C.c_void_p]
    C.CDLL(None).free(C.cast(out, C.c_void_p))
    return data


def write_particles_bin_reference(ids, member_off, member, halo_npart, order, minpart: int) -> bytes:
    """The reference's own binary writer (ahf_io_WriteParticles of the
    -DAHFbinary build), the AHF_particles_bin file read back."""
    return _writer(ref_bin_path(), "ahfref", ids, None, member_off, member, halo_npart, order, minpart, True)


def sfc_keys_oracle(x, y, z, bits: int = 21):
    """Restated Hilbert keys of float positions (sfc_curve_calcKey)."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_sfc_key
    fn.argtypes = [C.c_double, C.c_double, C.c_double, C.c_uint]
    fn.restype = C.c_uint64
    return np.array([fn(float(a), float(b), float(c), bits) for a, b, c in zip(x, y, z)], dtype=np.uint64)


def _sfc_sort(lib, name, x, y, z, extra):
    import numpy as np
    fn = getattr(lib, name)
    fn.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p] + [C.c_uint] * len(extra) + [C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    keys = np.zeros(len(a[0]), np.uint64)
    order = np.zeros(len(a[0]), np.uint64)
    if fn(len(a[0]), *[v.ctypes.data for v in a], *extra, keys.ctypes.data, order.ctypes.data) != 0:
        raise RuntimeError(f"{name} failed")
    return keys, order


def sfc_sort_oracle(x, y, z, bits: int = 21):
    """(keys ascending, original index of each): the restated keying and
    sort of main.c:342-356, equal keys by original index."""
    return _sfc_sort(C.CDLL(oracle_path()), "ahforacle_sfc_sort", x, y, z, [bits])


def sfc_sort_reference(x, y, z):
    """The reference's own keying (sfc_curve_calcKey, BITS_PER_DIMENSION) and
    qsort by cmp_sfckey_part."""
    return _sfc_sort(C.CDLL(ref_path(False)), "ahfref_sfc_sort", x, y, z, [])


def sfc_key_reference(x: float, y: float, z: float, bits: int) -> int:
    lib = C.CDLL(ref_path(False))
    fn = lib.ahfref_sfc_key
    fn.argtypes = [C.c_double, C.c_double, C.c_double, C.c_uint]
    fn.restype = C.c_uint64
    return int(fn(x, y, z, bits))


def ref_radii_path() -> str:
    return os.path.join(HERE, "_ref", "libahfref_radii.so")


def gather_radii_reference(npart, cx, cy, cz, rvir, max_gather_rad_box: float):
    """The reference's own gather-radius loop, run through spatialRef2halos
    on a two-level refinement tree (oracle/ref_radii.c).  Halo 0 is the
    tree's host, whose R_vir the reference leaves at -1: returns (radii,
    R_vir each halo carried)."""
    import numpy as np
    lib = C.CDLL(ref_radii_path())
    fn = lib.ahfref_gather_radii
    fn.argtypes = [C.c_int64] + [C.c_void_p] * 5 + [C.c_double, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    a = [np.ascontiguousarray(npart, dtype=np.uint64)] + [np.ascontiguousarray(v, dtype=np.float64)
                                                          for v in (cx, cy, cz, rvir)]
    n = len(a[0])
    rad = np.zeros(n)
    rv = np.zeros(n)
    rc = fn(n, *[v.ctypes.data for v in a], float(max_gather_rad_box), rad.ctypes.data, rv.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"ahfref_gather_radii failed ({rc})")
    return rad, rv


def ref_amr_path() -> str:
    return os.path.join(HERE, "_ref", "libahfref_amr.so")


_AMR_CHILD = r"""
import ctypes as C, json, sys
import numpy as np
a = np.load(sys.argv[1])
lib = C.CDLL(sys.argv[2])
f = lib.ahfref_amr_levels
f.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_int]
f.restype = C.c_int
x, y, z = (np.ascontiguousarray(a[k], dtype=np.float32) for k in ("x", "y", "z"))
lv = np.zeros(3 * 64, np.int64)
import time
t0 = time.perf_counter()
ng = f(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, int(a["ngrid_dom"]), int(a["ngrid_max"]),
       float(a["nth_dom"]), float(a["nth_ref"]), lv.ctypes.data, 64)
dt = time.perf_counter() - t0
print(json.dumps({"ngrids": int(ng), "levels": lv[:3 * max(ng, 0)].tolist(), "seconds": dt}))
"""


def amr_levels_reference(x, y, z, ngrid_dom: int, ngrid_max: int, nth_dom: float, nth_ref: float,
                         timed: bool = False):
    """The reference's own AMR hierarchy (gen_domgrids, ll, assign_npart,
    gen_AMRhierarchy; oracle/ref_amr.c) on float positions: an (ngrids, 3)
    int64 array of (l1dim, nodes, particles) per grid, and with `timed` also
    the seconds the call took (measured inside the child).  Runs in a child
    process: the hierarchy lives in the reference's globals until exit."""
    import json
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "in.npz")
        np.savez(path, x=np.asarray(x, np.float32), y=np.asarray(y, np.float32), z=np.asarray(z, np.float32),
                 ngrid_dom=ngrid_dom, ngrid_max=ngrid_max, nth_dom=nth_dom, nth_ref=nth_ref)
        r = subprocess.run([sys.executable, "-c", _AMR_CHILD, path, ref_amr_path()], capture_output=True, text=True,
                           check=True)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    if out["ngrids"] < 1:
        raise RuntimeError(f"ahfref_amr_levels failed ({out['ngrids']})")
    lv = np.array(out["levels"], dtype=np.int64).reshape(-1, 3)
    return (lv, float(out["seconds"])) if timed else lv


def domain_dens_oracle(x, y, z, l1: int):
    """Restated TSC densities of the l1^3 domain grid (assign_npart), as an
    (l1, l1, l1) array indexed [z, y, x]."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_domain_dens
    fn.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    fn.restype = C.c_int
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    out = np.zeros(l1 ** 3)
    if fn(len(a[0]), *[v.ctypes.data for v in a], int(l1), out.ctypes.data) != 0:
        raise RuntimeError("ahforacle_domain_dens failed")
    return out.reshape(l1, l1, l1)


_DENS_CHILD = r"""
import ctypes as C, sys
import numpy as np
a = np.load(sys.argv[1])
lib = C.CDLL(sys.argv[2])
f = lib.ahfref_domain_dens
f.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_void_p]
f.restype = C.c_int64
x, y, z = (np.ascontiguousarray(a[k], dtype=np.float32) for k in ("x", "y", "z"))
l1 = int(a["l1"])
out = np.zeros(l1 ** 3)
import time
t0 = time.perf_counter()
n = f(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, l1, out.ctypes.data)
dt = time.perf_counter() - t0
if n != l1 ** 3:
    sys.exit(3)
np.save(sys.argv[3], out)
open(sys.argv[3] + ".time", "w").write(repr(dt))
"""


def domain_dens_reference(x, y, z, l1: int, timed: bool = False):
    """The reference's own domain-grid densities after assign_npart
    (oracle/ref_amr.c), [z, y, x]; in a child process.  With `timed`, also
    the seconds the reference's calls took (gen_domgrids, ll, assign_npart,
    measured inside the child)."""
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "in.npz")
        np.savez(path, x=np.asarray(x, np.float32), y=np.asarray(y, np.float32), z=np.asarray(z, np.float32), l1=l1)
        subprocess.run([sys.executable, "-c", _DENS_CHILD, path, ref_amr_path(), os.path.join(d, "out.npy")],
                       check=True, capture_output=True)
        dens = np.load(os.path.join(d, "out.npy")).reshape(l1, l1, l1)
        if timed:
            return dens, float(open(os.path.join(d, "out.npy.time")).read())
        return dens


_REF1_CHILD = r"""
import ctypes as C, sys
import numpy as np
a = np.load(sys.argv[1])
lib = C.CDLL(sys.argv[2])
f = lib.ahfref_first_refinement
f.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_int64]
f.restype = C.c_int64
x, y, z = (np.ascontiguousarray(a[k], dtype=np.float32) for k in ("x", "y", "z"))
mx = 8 * int(a["dom"]) ** 3
out = np.zeros(3 * mx, np.int64)
k = f(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, int(a["dom"]), float(a["nd"]), float(a["nr"]),
      out.ctypes.data, mx)
if k < 0:
    sys.exit(3)
np.save(sys.argv[3], out[:3 * k].reshape(-1, 3))
"""


def first_refinement_reference(x, y, z, ngrid_dom: int, nth_dom: float, nth_ref: float):
    """The nodes (z, y, x in fine-grid units, quad order) of the first grid
    the reference refines from the ngrid_dom^3 domain grid (oracle/ref_amr.c);
    in a child process."""
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "in.npz")
        np.savez(path, x=np.asarray(x, np.float32), y=np.asarray(y, np.float32), z=np.asarray(z, np.float32),
                 dom=ngrid_dom, nd=nth_dom, nr=nth_ref)
        subprocess.run([sys.executable, "-c", _REF1_CHILD, path, ref_amr_path(), os.path.join(d, "out.npy")],
                       check=True, capture_output=True)
        return np.load(os.path.join(d, "out.npy"))


def first_refinement_oracle(x, y, z, l1: int, nth_dom: float):
    """Restated first refinement of the l1^3 domain grid: its fine nodes
    (z, y, x), ascending; empty when no grid is kept."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_first_refinement
    fn.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_int64]
    fn.restype = C.c_int64
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    mx = 8 * l1 ** 3
    out = np.zeros(3 * mx, np.int64)
    k = fn(len(a[0]), *[v.ctypes.data for v in a], int(l1), float(nth_dom), out.ctypes.data, mx)
    if k < 0:
        raise RuntimeError(f"ahforacle_first_refinement failed ({k})")
    return out[:3 * k].reshape(-1, 3)


def amr_levels_oracle(x, y, z, ngrid_dom: int, ngrid_max: int, nth_dom: float, nth_ref: float):
    """Restated AMR hierarchy (oracle_amr.c): (ngrids, 3) int64 array of
    (l1dim, nodes, particles) per grid."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_amr_levels
    fn.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                   C.c_void_p, C.c_int]
    fn.restype = C.c_int
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    lv = np.zeros(3 * 40, np.int64)
    ng = fn(len(a[0]), *[v.ctypes.data for v in a], int(ngrid_dom), int(ngrid_max), float(nth_dom), float(nth_ref),
            lv.ctypes.data, 40)
    if ng < 1:
        raise RuntimeError(f"ahforacle_amr_levels failed ({ng})")
    return lv[:3 * ng].reshape(-1, 3)


def _amr_nodes_call(lib, name, x, y, z, dom, mx, nd, nr, level):
    import numpy as np
    fn = getattr(lib, name)
    fn.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                                      C.c_void_p, C.c_void_p, C.c_int64]
    fn.restype = C.c_int64
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    mxn = 1 << 24
    zyx = np.zeros(3 * mxn, np.int64)
    dens = np.zeros(mxn)
    k = fn(len(a[0]), *[v.ctypes.data for v in a], int(dom), int(mx), float(nd), float(nr), int(level),
           zyx.ctypes.data, dens.ctypes.data, mxn)
    if k < 0:
        raise RuntimeError(f"{name} failed ({k})")
    return zyx[:3 * k].reshape(-1, 3), dens[:k]


def amr_nodes_oracle(x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, level: int):
    """Grid `level` of the restated hierarchy: (nodes (z, y, x), densities)."""
    return _amr_nodes_call(C.CDLL(oracle_path()), "ahforacle_amr_nodes", x, y, z, ngrid_dom, ngrid_max, nth_dom,
                           nth_ref, level)


def amr_all_nodes_oracle(x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, max_total: int = 1 << 26):
    """Every grid of the restated hierarchy from one build: a list of
    (nodes (z, y, x), densities) per grid."""
    import numpy as np
    fn = C.CDLL(oracle_path()).ahforacle_amr_all_nodes
    fn.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p,
                                                      C.c_void_p, C.c_int64, C.c_void_p, C.c_int]
    fn.restype = C.c_int
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    zyx = np.zeros(3 * max_total, np.int64)
    dens = np.zeros(max_total)
    counts = np.zeros(40, np.int64)
    ng = fn(len(a[0]), *[v.ctypes.data for v in a], int(ngrid_dom), int(ngrid_max), float(nth_dom), float(nth_ref),
            zyx.ctypes.data, dens.ctypes.data, max_total, counts.ctypes.data, 40)
    if ng < 1:
        raise RuntimeError(f"ahforacle_amr_all_nodes failed ({ng})")
    out, at = [], 0
    for g in range(ng):
        k = int(counts[g])
        out.append((zyx[3 * at:3 * (at + k)].reshape(-1, 3), dens[at:at + k]))
        at += k
    return out


_NODES_CHILD = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, sys.argv[4])
import oracle as O
a = np.load(sys.argv[1])
zyx, dens = O._amr_nodes_call(C.CDLL(sys.argv[2]), "ahfref_amr_nodes", a["x"], a["y"], a["z"], int(a["dom"]),
                              int(a["mx"]), float(a["nd"]), float(a["nr"]), int(a["level"]))
np.savez(sys.argv[3], zyx=zyx, dens=dens)
"""


def amr_nodes_reference(x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref, level: int):
    """Grid `level` of the reference's own hierarchy (oracle/ref_amr.c):
    (nodes (z, y, x) in quad order, densities); in a child process."""
    import sys
    import tempfile
    import numpy as np
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "in.npz")
        np.savez(path, x=np.asarray(x, np.float32), y=np.asarray(y, np.float32), z=np.asarray(z, np.float32),
                 dom=ngrid_dom, mx=ngrid_max, nd=nth_dom, nr=nth_ref, level=level)
        out = os.path.join(d, "out.npz")
        subprocess.run([sys.executable, "-c", _NODES_CHILD, path, ref_amr_path(), out, HERE], check=True,
                       capture_output=True)
        r = np.load(out)
        return r["zyx"], r["dens"]


def amr_list_order_violations(x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref) -> int:
    """Out-of-order pairs in the restated hierarchy's particle lists against
    index order, descending on even grids and ascending on odd ones."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_amr_list_order_violations
    fn.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_double, C.c_double]
    fn.restype = C.c_int64
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    return int(fn(len(a[0]), *[v.ctypes.data for v in a], int(ngrid_dom), int(ngrid_max), float(nth_dom),
                  float(nth_ref)))


def amr_gather_mismatches(x, y, z, ngrid_dom, ngrid_max, nth_dom, nth_ref) -> int:
    """Nodes, over all grids of the restated hierarchy, whose density
    computed as a gather (targets in order, sources in node order, particles
    in list order) differs from the reference-ordered scatter."""
    import numpy as np
    lib = C.CDLL(oracle_path())
    fn = lib.ahforacle_amr_gather_mismatches
    fn.argtypes = [C.c_uint64] + [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_double, C.c_double]
    fn.restype = C.c_int64
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
    return int(fn(len(a[0]), *[v.ctypes.data for v in a], int(ngrid_dom), int(ngrid_max), float(nth_dom),
                  float(nth_ref)))
