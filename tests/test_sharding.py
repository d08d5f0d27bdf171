"""Halo sharding across ranks (the multi-GPU path).

The split is the library's (ahfgpu_shard_halos), checked against an
independent statement of LPT.  On CPU, two gloo ranks run the oracle on their
shares; on the GPU, two ranks (two processes sharing cuda:0, each running
its own share with no wait on the other) call the library, rank 0 gathers
and merges; either way the merged result equals one process's bit for
bit."""
import os

import numpy as np
import pytest


def _lpt_statement(sizes, nranks):
    """Independent statement of the split: haloes by decreasing n log2(n+2)
    (stable), each to the least-loaded rank (ties: lower rank)."""
    import heapq
    cost = np.asarray(sizes, np.float64) * np.log2(np.asarray(sizes, np.float64) + 2.0)
    heap = [(0.0, r) for r in range(nranks)]
    out = np.zeros(len(sizes), np.int64)
    for h in np.argsort(-cost, kind="stable"):
        load, r = heapq.heappop(heap)
        out[h] = r
        heapq.heappush(heap, (load + cost[h], r))
    return out


def test_library_split_equals_lpt_statement():
    from ahf_gb300.shard import lpt_assign
    rng = np.random.default_rng(3)
    for nranks in (1, 2, 3, 8):
        sizes = np.floor(20 * (1 - rng.random(20000)) ** (-1 / 0.56)).astype(np.int64)
        sizes[:50] = 100   # equal costs: ties by index
        sizes[50:60] = 0   # empty lists
        assert np.array_equal(lpt_assign(sizes, nranks), _lpt_statement(sizes, nranks))
    assert len(lpt_assign(np.zeros(0, np.int64), 4)) == 0


def test_library_split_rejects_bad_offsets():
    import ctypes as C
    from ahf_gb300 import abi, lib
    off = np.array([0, 5, 3], np.uint64)
    out = np.zeros(2, np.int32)
    assert lib.load().ahfgpu_shard_halos(2, off.ctypes.data, 2, out.ctypes.data) == abi.AHFGPU_ERR_INVALID
    assert lib.load().ahfgpu_shard_halos(2, off.ctypes.data, 0, out.ctypes.data) == abi.AHFGPU_ERR_INVALID
    del C


def test_lpt_assign_balances_and_covers():
    from ahf_gb300.shard import lpt_assign
    rng = np.random.default_rng(1)
    sizes = np.floor(20 * (1 - rng.random(5000)) ** (-1 / 0.56)).astype(np.int64)
    r = lpt_assign(sizes, 4)
    assert set(np.unique(r)) == {0, 1, 2, 3}
    cost = sizes * np.log2(sizes + 2.0)
    loads = np.array([cost[r == k].sum() for k in range(4)])
    assert loads.max() <= loads.mean() + cost.max() + 1e-9


def _worker(rank, world, port, path, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path[:0] = [os.path.dirname(path), os.path.join(os.path.dirname(path), "oracle")]
    import oracle as O
    from ahf_gb300 import synth
    from ahf_gb300.shard import shard
    L = synth.generate("cfg4", scale=0.004)
    params = synth.params_for(L)
    sub, idx = shard(L, rank, world)
    res = O.run_oracle(params, sub)
    gathered = [None] * world
    dist.all_gather_object(gathered, (idx, res))
    if rank == 0:
        q.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shard_merge_equals_single_process(oracle_built):
    import socket

    import torch.multiprocessing as mp
    from ahf_gb300 import synth
    from ahf_gb300.shard import merge
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    procs = [ctx.Process(target=_worker, args=(r, 2, port, os.path.join(root, "bench.py"), q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    L = synth.generate("cfg4", scale=0.004)
    full = oracle_built.run_oracle(synth.params_for(L), L)
    merged = merge(gathered, L.nhalo)
    assert np.array_equal(merged["member_off"], full.member_off)
    assert np.array_equal(merged["member"], full.member)
    assert np.array_equal(merged["prof"], full.prof)
    assert np.array_equal(merged["halo_M_vir"], full.halo["M_vir"])
    assert all(len(g[0]) > 0 for g in gathered)


def _gpu_worker(rank, world, port, root, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path[:0] = [root]
    from ahf_gb300 import lib, synth
    from ahf_gb300.shard import shard
    lib.init(0)
    L = synth.generate("cfg3", scale=0.003, max_particles=60000)
    sub, idx = shard(L, rank, world)
    res = lib.construct_halos(synth.params_for(L), sub, "batched_fp32c")
    gathered = [None] * world
    dist.all_gather_object(gathered, (idx, res))
    if rank == 0:
        q.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_rank_library_shard_merge_equals_one_call():
    import socket

    import torch.multiprocessing as mp
    from ahf_gb300 import build, lib, synth
    from ahf_gb300.shard import merge
    build.build()
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    procs = [ctx.Process(target=_gpu_worker, args=(r, 2, port, root, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    L = synth.generate("cfg3", scale=0.003, max_particles=60000)
    lib.init(0)
    full = lib.construct_halos(synth.params_for(L), L, "batched_fp32c")
    merged = merge(gathered, L.nhalo)
    assert all(len(g[0]) > 0 for g in gathered)
    assert np.array_equal(merged["member_off"], full.member_off)
    assert np.array_equal(merged["member"], full.member)
    assert np.array_equal(merged["prof"], full.prof)
    for k in ("M_vir", "R_vir", "V2_max", "lambda_", "Phi0"):
        assert np.array_equal(merged["halo_" + k], full.halo[k]), k
