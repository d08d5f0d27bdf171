"""The AHF_particles writers: WriteParticlesLegacy (src/libahf/ahf_io.c:
1095-1175, ASCII) and ahf_binwrite_particles (:1733-1855, the AHFbinary
build's AHF_particles_bin).

CPU: the restated writers (oracle/ahf_oracle.c) byte-identical to the
reference's own -- the committed fixture tests/golden/writer_cfg1.npz
(`data`, `data_bin`) and, where the reference was compiled here, live on a
default, a MULTIMASS and an AHFbinary build.  GPU:
ahfgpu_write_particles_device / ahfgpu_write_particles_bin_device on a
device-resident stage result, byte-identical to the restated writers on the
same kept lists, and to the fixture when the stage runs on the fixture's
haloes.  Bar: identical bytes.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "writer_cfg1.npz")


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle
    oracle.build(ref=False)
    return oracle


def test_writer_restatement_matches_reference_fixture():
    O = _oracle()
    d = np.load(FIXTURE)
    got = O.write_particles_oracle(d["ids"], None, d["member_off"], d["member"], d["npart"], d["order"],
                                   int(d["minpart"]))
    assert got == d["data"].tobytes()


@pytest.mark.parametrize("multimass", [False, True])
def test_writer_restatement_matches_reference_live(multimass):
    O = _oracle()
    if not os.path.isfile(O.ref_path(multimass)):
        pytest.skip("reference not compiled here")
    from ahf_gb300 import synth
    L = (synth.generate("cfg3", scale=0.0005, max_particles=3000, multimass=True) if multimass
         else synth.generate("cfg4", scale=0.001))
    res = O.run_oracle(synth.params_for(L), L, 0)
    ids = np.arange(L.n, dtype=np.uint64) * np.uint64(3) + np.uint64(2**40)
    order = np.argsort(-res.halo["npart"].astype(np.int64), kind="stable")
    a = O.write_particles_oracle(ids, L.w, res.member_off, res.member, res.halo["npart"], order, 20)
    b = O.write_particles_reference(ids, L.w, res.member_off, res.member, res.halo["npart"], order, 20)
    assert a == b


def test_bin_writer_restatement_matches_reference_fixture():
    O = _oracle()
    d = np.load(FIXTURE)
    got = O.write_particles_bin_oracle(d["ids"], d["member_off"], d["member"], d["npart"], d["order"],
                                       int(d["minpart"]))
    assert got == d["data_bin"].tobytes()


def test_bin_writer_layout():
    """Header and block layout read back field by field."""
    O = _oracle()
    d = np.load(FIXTURE)
    b = O.write_particles_bin_oracle(d["ids"], d["member_off"], d["member"], d["npart"], d["order"], 20)
    good = [j for j, i in enumerate(d["order"]) if d["npart"][i] >= 20]
    assert np.frombuffer(b[:4], "<i4")[0] == 1
    assert np.frombuffer(b[4:12], "<u8")[0] == len(good)
    assert np.frombuffer(b[12:16], "<u4")[0] == 2
    pos = 16
    for j in good:
        i = d["order"][j]
        n, hj = np.frombuffer(b[pos:pos + 16], "<u8")
        assert (n, hj) == (d["npart"][i], j)
        rec = np.frombuffer(b[pos + 16:pos + 16 + 12 * n], np.dtype([("id", "<u8"), ("t", "<i4")]))
        mem = d["member"][d["member_off"][i]:d["member_off"][i] + n]
        assert np.array_equal(rec["id"], d["ids"][mem]) and np.all(rec["t"] == 1)
        pos += 16 + 12 * int(n)
    assert pos == len(b)


@pytest.mark.parametrize("minpart", [0, 20, 10**9])
def test_bin_writer_restatement_matches_reference_live(minpart):
    O = _oracle()
    if not os.path.isfile(O.ref_bin_path()):
        pytest.skip("reference not compiled here")
    from ahf_gb300 import synth
    L = synth.generate("cfg3", scale=0.0005, max_particles=3000, multimass=True)
    res = O.run_oracle(synth.params_for(L), L, 0)
    ids = np.arange(L.n, dtype=np.uint64) * np.uint64(5) + np.uint64(2**50)
    order = np.argsort(-res.halo["npart"].astype(np.int64), kind="stable")
    a = O.write_particles_bin_oracle(ids, res.member_off, res.member, res.halo["npart"], order, minpart)
    b = O.write_particles_bin_reference(ids, res.member_off, res.member, res.halo["npart"], order, minpart)
    assert a == b


@pytest.fixture(scope="module")
def gpu():
    from ahf_gb300 import build, lib
    build.build()
    lib.init(0)
    return lib


def _device_lists(L):
    import torch
    t = {"off": torch.as_tensor(L.off.astype(np.int64)).cuda()}
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        t[k] = torch.as_tensor(getattr(L, k)).cuda()
    t["w"] = torch.as_tensor(L.w).cuda() if L.w is not None else None
    t["gidx"] = torch.as_tensor(L.gidx.astype(np.int64)).cuda()
    for k in ("cx", "cy", "cz"):
        t[k] = torch.as_tensor(getattr(L, k)).cuda()
    torch.cuda.synchronize()
    return t


def _gpu_bytes(lib, ids, w, order, minpart):
    import torch
    addr, nb = lib.write_particles_device(ids, w, order, minpart)
    return lib.device_view(addr, nb, "|u1").cpu().numpy().tobytes() if nb else b""


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cfg4", "multimass", "large"])
def test_gpu_writer_matches_restatement(gpu, case):
    """Blocks of one and of several 4096-line chunks, MINPART 20 and 0."""
    import torch
    from ahf_gb300 import synth
    O = _oracle()
    L = (synth.generate("cfg3", scale=0.002, max_particles=20000, multimass=True) if case == "multimass"
         else synth.generate("cfg3", scale=0.0003, max_particles=300000) if case == "large"
         else synth.generate("cfg4", scale=0.01))
    t = _device_lists(L)
    gpu.construct_halos_device(synth.params_for(L), gpu.device_batch(t), "batched_fp32c")
    res = gpu.fetch_result()
    ids = np.arange(L.n, dtype=np.uint64) * np.uint64(977) + np.uint64(123456789)
    order = np.argsort(-res.halo["npart"].astype(np.int64), kind="stable").astype(np.int64)
    ids_d = torch.as_tensor(ids.astype(np.int64)).cuda()
    order_d = torch.as_tensor(order).cuda()
    for minpart in (20, 0):
        exp = O.write_particles_oracle(ids, L.w, res.member_off, res.member, res.halo["npart"], order, minpart)
        assert _gpu_bytes(gpu, ids_d, t["w"], order_d, minpart) == exp


@pytest.mark.gpu
def test_gpu_stage_and_writer_match_reference_fixture(gpu):
    """The fixture's haloes (cfg1) through the GPU stage (FP64,
    bit-exact kept lists) and the GPU writer: the reference's file."""
    import torch
    from ahf_gb300 import synth
    d = np.load(FIXTURE)
    L = synth.generate("cfg1")
    t = _device_lists(L)
    gpu.construct_halos_device(synth.params_for(L), gpu.device_batch(t), "batched_fp64")
    got = _gpu_bytes(gpu, torch.as_tensor(d["ids"].astype(np.int64)).cuda(), None,
                     torch.as_tensor(d["order"]).cuda(), int(d["minpart"]))
    assert got == d["data"].tobytes()


def _gpu_bin_bytes(lib, ids, order, minpart):
    addr, nb = lib.write_particles_bin_device(ids, order, minpart)
    return lib.device_view(addr, nb, "|u1").cpu().numpy().tobytes() if nb else b""


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cfg4", "multimass", "large"])
def test_gpu_bin_writer_matches_restatement(gpu, case):
    """Includes lists longer than one 4096-particle chunk ("large") and
    minpart 0 (haloes the stage left below MINPART are written too)."""
    import torch
    from ahf_gb300 import synth
    O = _oracle()
    L = (synth.generate("cfg3", scale=0.002, max_particles=20000, multimass=True) if case == "multimass"
         else synth.generate("cfg3", scale=0.0003, max_particles=300000) if case == "large"
         else synth.generate("cfg4", scale=0.01))
    t = _device_lists(L)
    gpu.construct_halos_device(synth.params_for(L), gpu.device_batch(t), "batched_fp32c")
    res = gpu.fetch_result()
    ids = np.arange(L.n, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15 % 2**40) + np.uint64(2**63 - 2**41)
    order = np.argsort(-res.halo["npart"].astype(np.int64), kind="stable").astype(np.int64)
    assert case != "large" or res.halo["npart"].max() > 3 * 4096
    ids_d = torch.as_tensor(ids.view(np.int64)).cuda()
    order_d = torch.as_tensor(order).cuda()
    for minpart in (20, 0):
        exp = O.write_particles_bin_oracle(ids, res.member_off, res.member, res.halo["npart"], order, minpart)
        assert _gpu_bin_bytes(gpu, ids_d, order_d, minpart) == exp


@pytest.mark.gpu
def test_gpu_stage_and_bin_writer_match_reference_fixture(gpu):
    """The fixture's haloes (cfg1) through the GPU stage (FP64, bit-exact
    kept lists) and the GPU binary writer: the reference's _bin file."""
    import torch
    from ahf_gb300 import synth
    d = np.load(FIXTURE)
    L = synth.generate("cfg1")
    t = _device_lists(L)
    gpu.construct_halos_device(synth.params_for(L), gpu.device_batch(t), "batched_fp64")
    got = _gpu_bin_bytes(gpu, torch.as_tensor(d["ids"].astype(np.int64)).cuda(), torch.as_tensor(d["order"]).cuda(),
                         int(d["minpart"]))
    assert got == d["data_bin"].tobytes()
