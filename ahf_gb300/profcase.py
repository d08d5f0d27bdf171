"""Small, self-contained cases of the stage for profilers (ncu).

    python -m ahf_gb300.profcase small [mode]   # 3000 haloes of <= 512 particles
    python -m ahf_gb300.profcase medium [mode]  # 300 haloes of 2048..16384 particles
    python -m ahf_gb300.profcase big [mode]     # one halo of ~2e5 particles
    python -m ahf_gb300.profcase full [mode]    # the whole 1e5-halo workload
    python -m ahf_gb300.profcase gather [scale] # the particle gather, the lists of 1e5*scale haloes as a snapshot
    python -m ahf_gb300.profcase sfc [n]        # Hilbert keys and sort of n seeded uniform points (5e7)

Each runs the stage twice on a device-resident batch cut from the seeded
1e5-halo workload (cfg3) and prints the device time and diagnostics.
mode: batched_fp32c (default), batched_fp64, plain_fp64.
"""
from __future__ import annotations

import sys

import numpy as np


def subset(lists, halos):
    import torch
    halos = np.asarray(halos, np.int64)
    off = lists.off.astype(np.int64)
    cnt = off[halos + 1] - off[halos]
    noff = np.zeros(len(halos) + 1, np.int64)
    noff[1:] = np.cumsum(cnt)
    idx = torch.as_tensor(np.concatenate([np.arange(off[h], off[h + 1]) for h in halos]), device="cuda")
    t = {"off": torch.as_tensor(noff, device="cuda")}
    for k in ("x", "y", "z", "vx", "vy", "vz", "w", "gidx"):
        v = getattr(lists, k)
        t[k] = None if v is None else v[idx].contiguous()
    for k in ("cx", "cy", "cz"):
        t[k] = torch.as_tensor(getattr(lists, k)[halos], device="cuda")
    return t


def gather_case(scale: float = 0.05) -> None:
    import time
    import torch
    from . import lib, synth
    lib.init(0)
    L = synth.generate("cfg3", scale=scale, device="cuda", as_numpy=False)
    n = np.diff(L.off.astype(np.int64))
    dev = L.x.device
    hid = torch.repeat_interleave(torch.arange(len(n), device=dev), torch.as_tensor(n, device=dev))
    d2 = torch.zeros(len(hid), dtype=torch.float64, device=dev)
    for a, c in ((L.x, L.cx), (L.y, L.cy), (L.z, L.cz)):
        d = (a.double() - torch.as_tensor(c, device=dev)[hid]).abs()
        d2 += torch.where(d > 0.5, 1.0 - d, d) ** 2
    rad = torch.zeros(len(n), dtype=torch.float64, device=dev).scatter_reduce(0, hid, d2, "amax").sqrt()
    parts = {k: getattr(L, k) for k in ("x", "y", "z", "vx", "vy", "vz", "w")}
    cen = {"cx": torch.as_tensor(L.cx).cuda(), "cy": torch.as_tensor(L.cy).cuda(), "cz": torch.as_tensor(L.cz).cuda(),
           "rad": rad}
    ms = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b = lib.gather_device(parts, cen)
        ms.append((time.perf_counter() - t0) * 1e3)
    off, _ = lib.gathered_lists(b)
    print(f"gather: haloes {len(n)} particles {int(L.x.numel())} gathered {int(off[-1])} "
          f"ms per call {', '.join(f'{m:.1f}' for m in ms)}")


def sfc_case(n: int = 50_000_000) -> None:
    import torch
    from . import lib
    lib.init(0)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    x, y, z = (torch.rand(n, device="cuda", generator=g) for _ in range(3))
    ms = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        keys, order = lib.sfc_sort_device(x, y, z)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    ok = bool((keys[1:] >= keys[:-1]).all().item())
    print(f"sfc: points {n} ascending {ok} ms per call {', '.join(f'{m:.2f}' for m in ms)}")


def main(argv):
    from . import lib, synth
    which = argv[0] if argv else "small"
    if which == "gather":
        gather_case(float(argv[1]) if len(argv) > 1 else 0.05)
        return
    if which == "sfc":
        sfc_case(int(float(argv[1])) if len(argv) > 1 else 50_000_000)
        return
    mode = argv[1] if len(argv) > 1 else "batched_fp32c"
    lib.init(0)
    scale = 1.0 if which == "full" else 0.05
    L = synth.generate("cfg3", scale=scale, device="cuda", as_numpy=False)
    p = synth.params_for(L)
    n = np.diff(L.off.astype(np.int64))
    if which == "small":
        sel = np.nonzero(n <= 512)[0][:3000]
    elif which == "medium":
        sel = np.nonzero((n > 2048) & (n <= 16384))[0][:300]
    elif which == "big":
        sel = np.array([int(np.argmin(np.abs(n - 200000)))])
    else:
        sel = np.arange(len(n))
    db = lib.device_batch(subset(L, sel))
    for _ in range(2):
        r = lib.construct_halos_device(p, db, mode)
    res = lib.fetch_result()
    print(f"{which} {mode}: haloes {len(sel)} particles {int(n[sel].sum())} ms {r.stats.ms_device:.3f} "
          f"fix_rounds max {res.halo['fix_rounds'].max()} niter mean {res.halo['niter'].mean():.2f} "
          f"retests {r.stats.n_retest} exact_iterations {r.stats.n_replay_halos}")


if __name__ == "__main__":
    main(sys.argv[1:])
