"""Halo sharding across processes / GPUs (no data-path collective).

Haloes are independent in the stage (src/libahf/ahf_halos.c:504-510 runs
them in any order), so a snapshot's batch is split by halo: each rank gets a
set of haloes chosen by longest-processing-time-first on the estimated cost
n log n, runs the stage on its own GPU, and the host merges the per-rank
results back into batch order.  Only the merge crosses ranks.
"""
from __future__ import annotations

import numpy as np


def lpt_assign(sizes, nranks: int) -> np.ndarray:
    """Rank of every halo: LPT on cost n*log2(n+2), ties to the lower halo
    index and the lower rank (ahfgpu_shard_halos, the library's split)."""
    from . import lib
    sizes = np.asarray(sizes, dtype=np.int64)
    off = np.zeros(len(sizes) + 1, np.uint64)
    off[1:] = np.cumsum(sizes)
    rank = np.zeros(len(sizes), np.int32)
    lib.check(lib.load().ahfgpu_shard_halos(len(sizes), off.ctypes.data, int(nranks), rank.ctypes.data))
    return rank.astype(np.int64)


def shard(lists, rank: int, nranks: int):
    """(sub-batch, halo indices) of `rank`'s share of a HaloLists batch."""
    sizes = np.diff(lists.off.astype(np.int64))
    owner = lpt_assign(sizes, nranks)
    mine = np.nonzero(owner == rank)[0]
    return lists.select(mine), mine


def merge(parts, nhalo: int) -> dict:
    """Merge per-rank results [(halo indices, HostResult)] into batch order:
    dict with halo (structured array), member_off, member, prof_off, prof."""
    from .abi import HALO_DTYPE, PROF_NFIELDS
    halo = np.zeros(nhalo, dtype=HALO_DTYPE)
    mem = [None] * nhalo
    prof = [None] * nhalo
    for idx, res in parts:
        for k, h in enumerate(idx):
            halo[h] = res.halo[k]
            mem[h] = res.members(k)
            prof[h] = res.profile(k)
    moff = np.zeros(nhalo + 1, np.uint64)
    moff[1:] = np.cumsum([len(m) for m in mem])
    poff = np.zeros(nhalo + 1, np.uint64)
    poff[1:] = np.cumsum([len(p) for p in prof])
    member = np.concatenate(mem) if nhalo else np.zeros(0, np.uint64)
    rows = np.concatenate(prof) if nhalo else np.zeros((0, PROF_NFIELDS))
    out = {"member_off": moff, "member": member, "prof_off": poff, "prof": rows}
    for k in halo.dtype.names:
        out["halo_" + k] = halo[k]
    return out
