"""Python binding of libahfgpu.so (the C ABI in include/ahfgpu.h).

This is the host-side mirror of the reference's call site: one
``construct_halos`` call stands for the per-halo loop of
src/libahf/ahf_halos.c:504-510 (ahf_halos_sfc_constructHalo minus the
gather).  There is no CPU fallback: if the CUDA library cannot be loaded or
no sm_103 device is present, every call raises ``AhfGpuError``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .abi import Batch, HostResult, Params, Result, make_batch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("AHFGPU_LIB", os.path.join(HERE, "libahfgpu.so"))

SYMBOLS = [
    "ahfgpu_init", "ahfgpu_shutdown", "ahfgpu_construct_halos", "ahfgpu_construct_halos_device",
    "ahfgpu_fetch_result", "ahfgpu_result_free", "ahfgpu_last_error", "ahfgpu_version", "ahfgpu_tuning",
    "ahfgpu_gather_device", "ahfgpu_gather_radii_device", "ahfgpu_write_particles_device",
    "ahfgpu_write_particles_bin_device", "ahfgpu_sfc_sort_device", "ahfgpu_shard_halos",
    "ahfgpu_amr_domain_density_device", "ahfgpu_amr_first_refinement_device", "ahfgpu_amr_hierarchy_device",
    "ahfgpu_amr_grid_device",
]


class AhfGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ahfgpu error {code}: {msg}")
        self.code = code


_lib = None
_inited_device = None


def load(path: str = LIB_PATH):
    """Load the shared library (raises if it is missing: no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(path):
        raise AhfGpuError(abi.AHFGPU_ERR_STATE, f"{path} not built (run __graft_entry__.build())")
    lib = C.CDLL(path)
    lib.ahfgpu_init.argtypes = [C.c_int]
    lib.ahfgpu_init.restype = C.c_int
    lib.ahfgpu_shutdown.argtypes = []
    lib.ahfgpu_shutdown.restype = C.c_int
    lib.ahfgpu_construct_halos.argtypes = [C.POINTER(Params), C.POINTER(Batch), C.POINTER(Result), C.c_int]
    lib.ahfgpu_construct_halos.restype = C.c_int
    lib.ahfgpu_construct_halos_device.argtypes = [C.POINTER(Params), C.POINTER(Batch), C.POINTER(Result),
                                                  C.c_int, C.c_void_p]
    lib.ahfgpu_construct_halos_device.restype = C.c_int
    lib.ahfgpu_fetch_result.argtypes = [C.POINTER(Result)]
    lib.ahfgpu_fetch_result.restype = C.c_int
    lib.ahfgpu_result_free.argtypes = [C.POINTER(Result)]
    lib.ahfgpu_result_free.restype = None
    lib.ahfgpu_last_error.argtypes = [C.c_char_p, C.c_size_t]
    lib.ahfgpu_last_error.restype = C.c_int
    lib.ahfgpu_version.argtypes = []
    lib.ahfgpu_version.restype = C.c_char_p
    lib.ahfgpu_tuning.argtypes = [C.c_char_p, C.c_size_t]
    lib.ahfgpu_tuning.restype = C.c_int
    lib.ahfgpu_gather_device.argtypes = [C.POINTER(abi.Particles), C.POINTER(abi.Centres), C.POINTER(Batch),
                                         C.c_void_p]
    lib.ahfgpu_gather_device.restype = C.c_int
    lib.ahfgpu_gather_radii_device.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    lib.ahfgpu_gather_radii_device.restype = C.c_int
    lib.ahfgpu_write_particles_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                                  C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_void_p]
    lib.ahfgpu_write_particles_device.restype = C.c_int
    lib.ahfgpu_write_particles_bin_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_void_p),
                                                      C.POINTER(C.c_uint64), C.c_void_p]
    lib.ahfgpu_write_particles_bin_device.restype = C.c_int
    lib.ahfgpu_amr_domain_density_device.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                                     C.c_void_p, C.c_void_p]
    lib.ahfgpu_amr_domain_density_device.restype = C.c_int
    lib.ahfgpu_amr_first_refinement_device.argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_double, C.c_void_p,
                                                       C.c_int64, C.POINTER(C.c_int64), C.c_void_p]
    lib.ahfgpu_amr_first_refinement_device.restype = C.c_int
    lib.ahfgpu_amr_hierarchy_device.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                                C.c_double, C.c_double, C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                                C.c_void_p]
    lib.ahfgpu_amr_hierarchy_device.restype = C.c_int
    lib.ahfgpu_amr_grid_device.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                           C.c_void_p]
    lib.ahfgpu_amr_grid_device.restype = C.c_int
    lib.ahfgpu_shard_halos.argtypes = [C.c_int64, C.c_void_p, C.c_int32, C.c_void_p]
    lib.ahfgpu_shard_halos.restype = C.c_int
    lib.ahfgpu_sfc_sort_device.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    lib.ahfgpu_sfc_sort_device.restype = C.c_int
    _lib = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(1024)
    lib.ahfgpu_last_error(buf, len(buf))
    return buf.value.decode()


def check(rc: int) -> None:
    if rc != abi.AHFGPU_OK:
        raise AhfGpuError(rc, last_error())


def init(device: int = 0) -> None:
    global _inited_device
    lib = load()
    if _inited_device == device:
        return
    check(lib.ahfgpu_init(device))
    _inited_device = device


def shutdown() -> None:
    global _inited_device
    if _lib is not None:
        check(_lib.ahfgpu_shutdown())
    _inited_device = None


def mode_id(mode) -> int:
    return abi.MODES[mode] if isinstance(mode, str) else int(mode)


def construct_halos(params: Params, lists, mode="batched_fp64", device: int = 0) -> HostResult:
    """Host batch in, host result out (the drop-in call)."""
    init(device)
    lib = load()
    b, keep = make_batch(lists)
    r = Result()
    check(lib.ahfgpu_construct_halos(C.byref(params), C.byref(b), C.byref(r), mode_id(mode)))
    try:
        return HostResult(r)
    finally:
        lib.ahfgpu_result_free(C.byref(r))
        del keep


def construct_halos_raw(params: Params, batch: Batch, mode) -> Result:
    """Host-pointer call returning the library-owned Result (caller frees
    with free_result); used where the caller already holds a Batch."""
    lib = load()
    r = Result()
    check(lib.ahfgpu_construct_halos(C.byref(params), C.byref(batch), C.byref(r), mode_id(mode)))
    return r


def free_result(r: Result) -> None:
    load().ahfgpu_result_free(C.byref(r))


def device_batch(t: dict) -> Batch:
    """Batch of device pointers from torch CUDA tensors (keys of HaloLists)."""
    b = Batch()
    b.nhalo = int(t["off"].numel() - 1)

    def p(name, ct):
        v = t.get(name)
        return C.cast(C.c_void_p(v.data_ptr() if v is not None else None), C.POINTER(ct))

    b.off = p("off", C.c_uint64)
    for n in ("x", "y", "z", "vx", "vy", "vz", "w"):
        setattr(b, n, p(n, C.c_float))
    b.gidx = p("gidx", C.c_uint64)
    for n in ("cx", "cy", "cz"):
        setattr(b, n, p(n, C.c_double))
    return b


def construct_halos_device(params: Params, dbatch: Batch, mode, stream: int | None = None) -> Result:
    """Device batch in, device-resident result description out."""
    lib = load()
    r = Result()
    check(lib.ahfgpu_construct_halos_device(C.byref(params), C.byref(dbatch), C.byref(r), mode_id(mode),
                                            C.c_void_p(stream) if stream else None))
    return r


def fetch_result() -> HostResult:
    lib = load()
    r = Result()
    check(lib.ahfgpu_fetch_result(C.byref(r)))
    try:
        return HostResult(r)
    finally:
        lib.ahfgpu_result_free(C.byref(r))


def version() -> str:
    return load().ahfgpu_version().decode()


def tuning(device: int = 0) -> dict:
    """The FP32C size-class tuning in effect on the device (see ahfgpu_tuning)."""
    import json
    init(device)
    buf = C.create_string_buffer(1024)
    check(load().ahfgpu_tuning(buf, len(buf)))
    return json.loads(buf.value.decode())


def gather_device(parts: dict, centres: dict, stream: int | None = None) -> Batch:
    """The GPU gather (ahfgpu_gather_device) on torch CUDA tensors:
    parts {x, y, z, vx, vy, vz[, w]}, centres {cx, cy, cz, rad}.  Returns the
    gathered batch (device pointers, library-owned until the next gather),
    ready for construct_halos_device."""
    init()
    p = abi.Particles()
    p.n = int(parts["x"].numel())
    for k in ("x", "y", "z", "vx", "vy", "vz", "w"):
        v = parts.get(k)
        setattr(p, k, C.cast(C.c_void_p(v.data_ptr() if v is not None else None), C.POINTER(C.c_float)))
    c = abi.Centres()
    c.nhalo = int(centres["cx"].numel())
    for k in ("cx", "cy", "cz", "rad"):
        setattr(c, k, C.cast(C.c_void_p(centres[k].data_ptr()), C.POINTER(C.c_double)))
    b = Batch()
    check(load().ahfgpu_gather_device(C.byref(p), C.byref(c), C.byref(b), C.c_void_p(stream) if stream else None))
    return b


def device_view(ptr: int, count: int, typestr: str):
    """A torch CUDA tensor viewing `count` elements at a device address the
    library owns (no copy)."""
    import torch

    class _Dev:
        __cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (ptr, False), "version": 3}
    return torch.as_tensor(_Dev(), device="cuda")


def gathered_lists(b: Batch):
    """(off, gidx) of a gathered batch, copied to host numpy arrays."""
    import numpy as np
    import torch
    torch.cuda.synchronize()
    nh = int(b.nhalo)
    off = device_view(C.cast(b.off, C.c_void_p).value, nh + 1, "<u8").cpu().numpy().astype(np.uint64)
    n = int(off[-1])
    gid = (device_view(C.cast(b.gidx, C.c_void_p).value, n, "<u8").cpu().numpy().astype(np.uint64) if n
           else np.zeros(0, np.uint64))
    return off, gid


def gather_radii_device(npart, cx, cy, cz, rvir, max_gather_rad_box: float, stream: int | None = None):
    """ahfgpu_gather_radii_device on torch CUDA tensors; returns the radii
    (float64 CUDA tensor)."""
    import torch
    init()
    out = torch.empty(npart.numel(), dtype=torch.float64, device=npart.device)
    check(load().ahfgpu_gather_radii_device(int(npart.numel()), npart.data_ptr(), cx.data_ptr(), cy.data_ptr(),
                                           cz.data_ptr(), rvir.data_ptr(), float(max_gather_rad_box),
                                           out.data_ptr(), C.c_void_p(stream) if stream else None))
    return out


def write_particles_device(ids, w, order, minpart: int, stream: int | None = None):
    """ahfgpu_write_particles_device for the last device result; ids, w
    (or None), order are torch CUDA tensors.  Returns (device address,
    nbytes) of the AHF_particles bytes."""
    init()
    out = C.c_void_p()
    nb = C.c_uint64()
    check(load().ahfgpu_write_particles_device(ids.data_ptr(), w.data_ptr() if w is not None else None,
                                              order.data_ptr(), int(minpart), C.byref(out), C.byref(nb),
                                              C.c_void_p(stream) if stream else None))
    return out.value, nb.value


def write_particles_bin_device(ids, order, minpart: int, stream: int | None = None):
    """ahfgpu_write_particles_bin_device for the last device result; ids and
    order are torch CUDA tensors.  Returns (device address, nbytes) of the
    AHF_particles_bin bytes."""
    init()
    out = C.c_void_p()
    nb = C.c_uint64()
    check(load().ahfgpu_write_particles_bin_device(ids.data_ptr(), order.data_ptr(), int(minpart), C.byref(out),
                                                  C.byref(nb), C.c_void_p(stream) if stream else None))
    return out.value, nb.value


def sfc_sort_device(x, y, z, bits: int = 21, stream: int | None = None):
    """ahfgpu_sfc_sort_device on float32 CUDA tensors x, y, z: (keys, order)
    as int64 CUDA tensors (keys hold the uint64 Hilbert keys bit for bit)."""
    import torch
    init()
    n = int(x.numel())
    keys = torch.empty(n, dtype=torch.int64, device=x.device)
    order = torch.empty(n, dtype=torch.int64, device=x.device)
    check(load().ahfgpu_sfc_sort_device(n, x.data_ptr(), y.data_ptr(), z.data_ptr(), int(bits), keys.data_ptr(),
                                        order.data_ptr(), C.c_void_p(stream) if stream else None))
    return keys, order


def amr_domain_density_device(x, y, z, l1: int, stream: int | None = None):
    """TSC density minus the mean of the l1^3 domain grid (float, z-major)
    from device float positions (torch tensors)."""
    import torch
    lib = load()
    dens = torch.empty(l1 * l1 * l1, dtype=torch.float32, device=x.device)
    check(lib.ahfgpu_amr_domain_density_device(int(x.numel()), x.data_ptr(), y.data_ptr(), z.data_ptr(), int(l1),
                                               dens.data_ptr(), C.c_void_p(stream) if stream else None))
    return dens


def amr_first_refinement_device(dens, l1: int, n: int, nth_dom: float, stream: int | None = None):
    """(z, y, x) of the first refined grid's nodes (int32 [k, 3] on the
    device, ascending; empty below MIN_NNODES)."""
    import torch
    lib = load()
    cap = 8 * l1 * l1 * l1
    out = torch.empty((cap, 3), dtype=torch.int32, device=dens.device)
    nn = C.c_int64(0)
    check(lib.ahfgpu_amr_first_refinement_device(int(l1), dens.data_ptr(), int(n), float(nth_dom), out.data_ptr(),
                                                 cap, C.byref(nn), C.c_void_p(stream) if stream else None))
    return out[:nn.value]


def amr_hierarchy_device(x, y, z, ngrid_dom: int, ngrid_max: int, nth_dom: float, nth_ref: float,
                         stream: int | None = None) -> np.ndarray:
    """The whole AMR hierarchy from device float positions (torch tensors):
    an (ngrids, 3) int64 array of nodes per dimension, nodes and listed
    particles per grid.  The grids stay in the library for amr_grid_device."""
    lib = load()
    cap = 64
    lv = np.zeros(3 * cap, np.int64)
    ng = C.c_int(0)
    check(lib.ahfgpu_amr_hierarchy_device(int(x.numel()), x.data_ptr(), y.data_ptr(), z.data_ptr(), int(ngrid_dom),
                                          int(ngrid_max), float(nth_dom), float(nth_ref),
                                          lv.ctypes.data_as(C.c_void_p), cap, C.byref(ng),
                                          C.c_void_p(stream) if stream else None))
    return lv[:3 * ng.value].reshape(-1, 3)


def amr_grid_device(level: int, device="cuda", stream: int | None = None):
    """Grid `level` of the last hierarchy: (zyx int32 [k, 3], dens float32
    [k]) torch tensors on the device, in the reference's node order."""
    import torch
    lib = load()
    nn = C.c_int64(0)
    check(lib.ahfgpu_amr_grid_device(int(level), None, None, 0, C.byref(nn), None))
    k = nn.value
    zyx = torch.empty((max(k, 1), 3), dtype=torch.int32, device=device)
    dens = torch.empty(max(k, 1), dtype=torch.float32, device=device)
    if k:
        check(lib.ahfgpu_amr_grid_device(int(level), zyx.data_ptr(), dens.data_ptr(), k, C.byref(nn),
                                         C.c_void_p(stream) if stream else None))
    return zyx[:k], dens[:k]
