"""ahfgpu_construct_halos_noalloc against the allocating entry point.

The no-allocation entry point serves callers that cannot allocate device
memory (an application that partitions the GPU's memory itself and gives the
analysis a fixed budget, or a plugin inside a running simulation that may not
call cudaMalloc): its work space is one static device array, and the caller
passes device buffers for every input and output.  This test calls it through the C ABI twice in a
row on the same batch and checks both results against ahfgpu_construct_halos
in the batched FP64 form: identical kept lists, properties within 1e-10
relative, eigenvectors up to sign, with and without MULTIMASS weights.  It
also checks the size limits.  The
file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from compare import compare

pytestmark = pytest.mark.gpu


def _lib():
    from ahf_gb300 import build, lib
    build.build()
    lib.init(0)
    l = lib.load()
    l.ahfgpu_construct_halos_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p]
    l.ahfgpu_construct_halos_noalloc.restype = C.c_int
    l.ahfgpu_noalloc_last_error.argtypes = [C.c_char_p, C.c_size_t]
    l.ahfgpu_noalloc_last_error.restype = C.c_int
    return lib, l


def _noalloc_call(l, params, dbatch, nhalo, n):
    import torch
    from ahf_gb300 import abi
    maxb = 64   # AHFGPU_NOALLOC_MAX_BINS
    out_halo = torch.zeros(nhalo * C.sizeof(abi.Halo), dtype=torch.uint8, device="cuda")
    out_member = torch.zeros(max(n, 1), dtype=torch.int64, device="cuda")
    out_prof = torch.zeros(nhalo * maxb * abi.PROF_NFIELDS, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = l.ahfgpu_construct_halos_noalloc(C.addressof(params), C.addressof(dbatch), out_halo.data_ptr(),
                                          out_member.data_ptr(), out_prof.data_ptr(), None)
    if rc != 0:
        buf = C.create_string_buffer(256)
        l.ahfgpu_noalloc_last_error(buf, 256)
        raise AssertionError(f"noalloc rc={rc}: {buf.value.decode()}")
    torch.cuda.synchronize()
    halo = out_halo.cpu().numpy().view(abi.HALO_DTYPE).copy()
    mem = out_member.cpu().numpy().view(np.uint64)
    prof = out_prof.cpu().numpy().reshape(nhalo, maxb, abi.PROF_NFIELDS)
    return halo, mem, prof


def _pack(halo, mem, prof, off):
    """staging layout -> packed CSR result dict (the shape compare() reads)"""
    nh = len(halo)
    npart = halo["npart"].astype(np.int64)
    nb = halo["nbins"].astype(np.int64)
    moff = np.zeros(nh + 1, np.uint64)
    moff[1:] = np.cumsum(npart)
    poff = np.zeros(nh + 1, np.uint64)
    poff[1:] = np.cumsum(nb)
    members = np.concatenate([mem[int(off[h]):int(off[h]) + npart[h]] for h in range(nh)])
    rows = np.concatenate([prof[h, :nb[h]] for h in range(nh)]) if nb.sum() else np.zeros((0, prof.shape[2]))
    d = {"member_off": moff, "member": members, "prof_off": poff, "prof": rows}
    for k in halo.dtype.names:
        d["halo_" + k] = halo[k]
    return d


@pytest.mark.parametrize("multimass", [False, True])
def test_noalloc_matches_allocating_entry_point_twice(multimass):
    import torch
    from ahf_gb300 import synth
    lib, l = _lib()
    L = synth.generate("cfg3", scale=0.002, max_particles=12000, multimass=multimass)
    # keep the batch within the static work space
    n = np.diff(L.off.astype(np.int64))
    keep = np.nonzero(np.cumsum(n) <= 120000)[0]
    L = L.select(keep)
    params = synth.params_for(L)
    exp = lib.construct_halos(params, L, "batched_fp64")
    t = {"off": torch.as_tensor(L.off.astype(np.int64)).cuda()}
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        t[k] = torch.as_tensor(getattr(L, k)).cuda()
    if L.w is not None:
        t["w"] = torch.as_tensor(L.w).cuda()
    t["gidx"] = torch.as_tensor(L.gidx.astype(np.int64)).cuda()
    for k in ("cx", "cy", "cz"):
        t[k] = torch.as_tensor(getattr(L, k)).cuda()
    db = lib.device_batch(t)
    for call in range(2):
        halo, mem, prof = _noalloc_call(l, params, db, L.nhalo, L.n)
        got = _pack(halo, mem, prof, L.off)
        assert np.array_equal(got["member"], exp.member), f"call {call}: kept lists differ"
        bad = compare(got, exp, rtol=1e-10, etol=1e-8)
        assert not bad, (call, bad)


def test_noalloc_rejects_sizes_beyond_the_limits():
    import torch
    from ahf_gb300 import abi
    lib, l = _lib()
    from ahf_gb300 import synth
    L = synth.generate("cfg1", scale=0.2)
    params = synth.params_for(L)
    # too many haloes: rejected before any device work
    b = abi.Batch()
    b.nhalo = 8193
    rc = l.ahfgpu_construct_halos_noalloc(C.addressof(params), C.addressof(b), 1, 1, 1, None)
    assert rc == abi.AHFGPU_ERR_CAPACITY
    # too many particles: off[nhalo] beyond AHFGPU_NOALLOC_MAX_PARTICLES
    off = torch.as_tensor(np.array([0, 131073], np.int64)).cuda()
    z = torch.zeros(131073, dtype=torch.float32, device="cuda")
    c = torch.zeros(1, dtype=torch.float64, device="cuda")
    db = lib.device_batch({"off": off, "x": z, "y": z, "z": z, "vx": z, "vy": z, "vz": z,
                           "cx": c, "cy": c, "cz": c})
    torch.cuda.synchronize()
    rc = l.ahfgpu_construct_halos_noalloc(C.addressof(params), C.addressof(db), c.data_ptr(), c.data_ptr(),
                                          c.data_ptr(), None)
    assert rc == abi.AHFGPU_ERR_CAPACITY
