"""Halo sharding across ranks (the multi-GPU path, exercised on CPU with the
gloo backend and the oracle as the per-rank stage): two ranks each process
their LPT share, rank 0 gathers and merges, and the merged result equals the
single-process result bit for bit."""
import os

import numpy as np
import pytest


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
