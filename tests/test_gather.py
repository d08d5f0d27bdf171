"""The particle gather (ahf_halos_sfc_gatherParts, src/libahf/ahf_halos_sfc.c:171-412).

CPU: the gather restatement (oracle/ahf_oracle.c) against the reference's own
SFC gather -- the committed fixtures tests/golden/gather_*.npz and, where the
reference was compiled here, live runs.  GPU: ahfgpu_gather_device through the
C ABI against the restatement (lists identical, ascending particle index) and
against the fixtures (the same sets as the reference), and the gathered
batch through the stage against the oracle on the oracle's lists.
Bars: gathered lists identical; the stage's FP64 bars on top of the gather.
"""
import glob
import os
import sys

import numpy as np
import pytest

from compare import compare

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "gather_*.npz")))


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle
    oracle.build(ref=False)
    return oracle


def _sorted_lists(off, idx):
    return [np.sort(idx[int(off[h]):int(off[h + 1])]) for h in range(len(off) - 1)]


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gather_restatement_matches_reference_fixtures(path):
    O = _oracle()
    d = np.load(path)
    off, idx = O.gather_oracle(d["x"], d["y"], d["z"], d["cx"], d["cy"], d["cz"], d["rad"])
    assert np.array_equal(off, d["off"])
    for h, ref in enumerate(_sorted_lists(d["off"], d["idx"])):
        assert np.array_equal(idx[int(off[h]):int(off[h + 1])], ref), h


def test_gather_restatement_matches_reference_live():
    O = _oracle()
    if not os.path.isfile(O.ref_path(False)):
        pytest.skip("reference not compiled here")
    from ahf_gb300 import synth
    S = synth.snapshot_from_lists(synth.generate("cfg4", scale=0.002), 20000, seed=3)
    off, idx = O.gather_oracle(S.x, S.y, S.z, S.cx, S.cy, S.cz, S.rad)
    roff, ridx = O.gather_reference(S.x, S.y, S.z, S.cx, S.cy, S.cz, S.rad)
    assert np.array_equal(off, roff)
    for h, ref in enumerate(_sorted_lists(roff, ridx)):
        assert np.array_equal(idx[int(off[h]):int(off[h + 1])], ref), h


# ------------------------------------------------------------------ GPU
def _gpu_gather(S):
    import torch
    from ahf_gb300 import lib
    parts = {k: torch.as_tensor(np.ascontiguousarray(getattr(S, k))).cuda() for k in ("x", "y", "z", "vx", "vy", "vz")}
    parts["w"] = torch.as_tensor(S.w).cuda() if S.w is not None else None
    cen = {k: torch.as_tensor(np.ascontiguousarray(getattr(S, k), dtype=np.float64)).cuda()
           for k in ("cx", "cy", "cz", "rad")}
    torch.cuda.synchronize()
    b = lib.gather_device(parts, cen)
    off, gid = lib.gathered_lists(b)
    return b, (parts, cen), off, gid


@pytest.fixture(scope="module")
def gpu():
    from ahf_gb300 import build, lib
    build.build()
    lib.init(0)
    return lib


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gpu_gather_matches_reference_fixtures(gpu, path):
    from ahf_gb300 import synth
    d = np.load(path)
    S = synth.Snapshot(d["x"], d["y"], d["z"], d["x"] * 0, d["y"] * 0, d["z"] * 0, None, d["cx"], d["cy"], d["cz"],
                       d["rad"])
    _, _, off, gid = _gpu_gather(S)
    assert np.array_equal(off, d["off"])
    for h, ref in enumerate(_sorted_lists(d["off"], d["idx"])):
        got = gid[int(off[h]):int(off[h + 1])]
        assert np.array_equal(got, ref), h          # ascending index, the reference's set


@pytest.mark.gpu
def test_gpu_gather_matches_restatement(gpu):
    from ahf_gb300 import synth
    O = _oracle()
    S = synth.snapshot_from_lists(synth.generate("cfg4", scale=0.02), 500000, seed=5)
    _, _, off, gid = _gpu_gather(S)
    ooff, oidx = O.gather_oracle(S.x, S.y, S.z, S.cx, S.cy, S.cz, S.rad)
    assert np.array_equal(off, ooff)
    assert np.array_equal(gid, oidx)


def _packed(b, n):
    """The gathered batch's particle arrays (device) as host numpy arrays."""
    import ctypes as C
    from ahf_gb300 import lib
    out = {}
    for k in ("x", "y", "z", "vx", "vy", "vz", "w"):
        ptr = C.cast(getattr(b, k), C.c_void_p).value
        out[k] = lib.device_view(ptr, n, "<f4").cpu().numpy() if ptr and n else None
    return out


# The lists' order: per window of each list's index range, a bitmap where the
# window's keys are dense (lists of a snapshot in list order), a bitonic
# network where they are sparse (a shuffled snapshot), the block radial sort
# for lists the windows do not cover; the hooks force each path and narrow
# the window so that lists span many windows (queued as window items).
ORDER_CASES = [
    ("list_order", False, {}),
    ("shuffled", True, {}),
    ("list_order_fallback_only", False, {"AHFGPU_GATHER_BITMAP": "0"}),
    ("shuffled_bitmap_only_64bit_windows", True, {"AHFGPU_GATHER_BITMAP": "2", "AHFGPU_GATHER_WBITS": "64"}),
    ("list_order_256bit_windows", False, {"AHFGPU_GATHER_WBITS": "256"}),
    ("list_order_network_only", False, {"AHFGPU_GATHER_BITMAP": "3"}),
    ("shuffled_network_256bit_windows", True, {"AHFGPU_GATHER_BITMAP": "3", "AHFGPU_GATHER_WBITS": "256"}),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,shuffle,env", ORDER_CASES, ids=[c[0] for c in ORDER_CASES])
def test_gpu_gather_order_paths(gpu, name, shuffle, env, monkeypatch):
    from ahf_gb300 import synth
    O = _oracle()
    L = synth.generate("cfg4", scale=0.01, multimass=True)   # with a mass array, so that it is packed too
    S = synth.snapshot_from_lists(L, 200000, seed=13, shuffle=shuffle)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    b, _, off, gid = _gpu_gather(S)
    ooff, oidx = O.gather_oracle(S.x, S.y, S.z, S.cx, S.cy, S.cz, S.rad)
    assert np.array_equal(off, ooff)
    assert np.array_equal(gid, oidx)
    got = _packed(b, len(gid))
    sel = gid.astype(np.int64)
    for k in ("x", "y", "z", "vx", "vy", "vz", "w"):
        assert np.array_equal(got[k], np.asarray(getattr(S, k))[sel]), k


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched_fp64", "batched_fp32c"])
def test_gather_then_stage_matches_oracle(gpu, mode):
    """The gathered batch straight into the stage (device-resident), against
    the oracle stage on the restatement's lists."""
    from ahf_gb300 import lib, synth
    from compare import compare_fp32c
    O = _oracle()
    L = synth.generate("cfg1")
    S = synth.snapshot_from_lists(L, 60000, seed=9)
    b, keep, off, gid = _gpu_gather(S)
    params = synth.params_for(L)
    lib.construct_halos_device(params, b, mode)
    got = lib.fetch_result()
    ooff, oidx = O.gather_oracle(S.x, S.y, S.z, S.cx, S.cy, S.cz, S.rad)
    g = lambda a: None if a is None else np.ascontiguousarray(a[oidx.astype(np.int64)])
    lists = synth.HaloLists(ooff, g(S.x), g(S.y), g(S.z), g(S.vx), g(S.vy), g(S.vz), g(S.w), oidx.copy(),
                            S.cx, S.cy, S.cz, L.boxsize, L.pmass, "gathered")
    exp = O.run_oracle(params, lists, 0)
    bad = compare(got, exp, rtol=1e-10, etol=1e-8) if mode == "batched_fp64" else compare_fp32c(got, exp)
    assert not bad, bad
    assert np.array_equal(got.member, exp.member)
