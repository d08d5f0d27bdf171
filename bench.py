"""Benchmark of the unbinding + halo-property stage (one JSON line).

Workload (default): the 1e5-halo snapshot "cfg3" -- 1e5 particle lists with
N_p ~ N^-1.56 on [20, 2e6] (sum ~ 4e8), float32 positions/velocities, equal
masses, 64-bit ids -- generated seeded and synthetic on the GPU (AHF ships no
data).  A step is one call of the stage over the whole batch.

  value   particles/s with the batch resident in HBM (ahfgpu_construct_halos_
          device), CUDA events on the stream the library runs on
  e2e     the same through the host API ahfgpu_construct_halos with pinned
          host buffers: host->device copy of the particle lists and device->
          host copy of the kept lists, properties and profiles every step
  roofline  dominant kernel: algorithmic bytes per launch / its CUDA-event
          duration, against the measured HBM copy bandwidth
  cpu_baseline  the oracle (the reference's algorithm restated in C; the
          reference's own code where it was built) on all host cores, on a
          bounded sample of the same haloes

`--impl reference` times the reference's own routines (compiled from its
sources on the host; the C restatement where they could not be built) on all
host cores, its K timed steps together covering the whole workload (rank 0;
other ranks exit).  Under torchrun every rank builds the same batch and runs
its share of the haloes (the library's LPT split, ahfgpu_shard_halos): strong
scaling, no collective on the data path.

`--case small|medium|large|big|gather|sfc|amr` runs one small device-resident case
twice and prints its device time (the cases the profiles/ summaries were
captured on): 3000 lists of <= 512 entries, 300 of 2048-16384, the 160
lists nearest 1e5 entries of a 1.5e4-halo batch (about one per SM, as at full
load), one of ~2e5,
the gather on the lists of 5e3 haloes as a snapshot, the Hilbert sort of
5e7 uniform points, the AMR hierarchy of the 256^3-particle cfg2 box.
`--case phases` builds the library with -DAHFGPU_PHASE_TIMERS into a separate
file and prints the FP32C stage's SM cycles per list entry, phase by phase,
on the class-2 lists (more than 32768 entries) of the 1e5-halo batch.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particles unbound/s"
UNIT = "particles/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg3")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--mode", default=None, help="form timed for `value` (default: fastest built)")
    ap.add_argument("--forms", default="all", help="comma list of extra forms to time once, or none")
    ap.add_argument("--cpu-particles", type=float, default=6e7, help="CPU baseline sample size")
    ap.add_argument("--cpu-repeats", type=int, default=3, help="CPU baseline: best of this many runs")
    ap.add_argument("--cpu-serial-particles", type=float, default=5e6,
                    help="sample size of the one-thread CPU rate (0: skip)")
    ap.add_argument("--plain-particles", type=float, default=2e7, help="plain FP64 form sample size")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-gather", action="store_true", help="skip the particle-gather leg")
    ap.add_argument("--no-writer", action="store_true", help="skip the AHF_particles writer leg")
    ap.add_argument("--gather-cpu-particles", type=float, default=2e7, help="CPU gather baseline sample size")
    ap.add_argument("--no-sfc", action="store_true", help="skip the Hilbert key sort leg")
    ap.add_argument("--no-amr", action="store_true", help="skip the AMR hierarchy leg")
    ap.add_argument("--multimass", action="store_true")
    ap.add_argument("--case", default=None,
                    choices=["small", "medium", "large", "big", "gather", "sfc", "amr", "phases"],
                    help="run one small profiling case instead of the benchmark")
    ap.add_argument("--case-arg", type=float, default=None, help="gather: halo scale; sfc: points")
    return ap.parse_args()


# ---------------------------------------------------------------- helpers

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        # median over samples under load (upper half of the clock samples)
        s = np.sort(np.array(sm))
        load = s[len(s) // 2:] if len(s) > 3 else s
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": float(max(mx)), "samples": len(sm),
                "reasons": sorted(reasons)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload: str, kernel: str):
    """Per-particle DRAM traffic of the dominant kernel from the committed ncu
    summary (profiles/<kernel>_<workload>.md, line 'dram_bytes_per_particle: X')."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.isfile(p):
        return None
    for line in open(p):
        if line.strip().startswith("dram_bytes_per_particle:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def alg_bytes(n_in: np.ndarray, res_halo, has_w: bool) -> float:
    """Compulsory bytes of one call: pos+vel (+mass) read once per gathered
    particle, the 8-byte id of each kept particle read and written, the centre
    in, the profile rows and ~256 B of properties out."""
    nb = res_halo["npart"].astype(np.float64)
    nbins = res_halo["nbins"].astype(np.float64)
    per_p = 24.0 + (4.0 if has_w else 0.0)
    return float(per_p * n_in.sum() + 16.0 * nb.sum() + (24.0 + 256.0) * len(n_in) + 8.0 * 25.0 * nbins.sum())


def precision_report(r32, r64, retests, against: str) -> dict:
    """The FP32-compensated result `r32` against `r64` (the FP64 oracle or the
    batched FP64 form) on the same haloes: haloes whose kept lists differ
    (must be 0), the largest relative differences of Phi0, M_vir, R_vir,
    V_max = sqrt(V2_max), sigV and the spin lambda, and the particles routed
    to the FP64 re-test."""
    n = len(r32.halo)
    diff = 0
    m32, m64, o32, o64 = r32.member, r64.member, r32.member_off, r64.member_off
    if not np.array_equal(o32, o64):
        diff = int(np.count_nonzero(np.diff(o32.astype(np.int64)) != np.diff(o64.astype(np.int64))))
    elif not np.array_equal(m32, m64):
        bad = np.nonzero(m32 != m64)[0]
        diff = int(len(np.unique(np.searchsorted(o32.astype(np.int64), bad, side="right") - 1)))

    def rel(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        ok = np.isfinite(a) & np.isfinite(b) & (b != 0)
        return float(np.max(np.abs(a[ok] - b[ok]) / np.abs(b[ok]))) if ok.any() else 0.0
    h32, h64 = r32.halo, r64.halo
    prof = (h64["flags"] & 0x20) != 0   # AHFGPU_HALO_RAN_PROFILE
    l32, l64 = h32["lambda_"][prof].astype(np.float64), h64["lambda_"][prof].astype(np.float64)
    le = np.abs(l32 - l64) / np.maximum(np.abs(l64), 1e-300)
    iw = int(np.argmax(le)) if le.size else 0
    worst = ({"npart": int(h64["npart"][prof][iw]), "lambda": float(l64[iw]), "rel_err": float(le[iw]),
              "median_lambda": float(np.median(np.abs(l64))), "haloes_above_1e-6": int(np.sum(le > 1e-6))}
             if le.size else None)
    return {"haloes": n, "particles": int(o64[-1]) if len(o64) else 0, "kept_list_mismatches": diff,
            "lambda_worst": worst, "max_rel_err": {
                "Phi0": rel(h32["Phi0"], h64["Phi0"]), "M_vir": rel(h32["M_vir"], h64["M_vir"]),
                "R_vir": rel(h32["R_vir"], h64["R_vir"]),
                "V_max": rel(np.sqrt(np.abs(h32["V2_max"][prof])), np.sqrt(np.abs(h64["V2_max"][prof]))),
                "sigV": rel(h32["sigV"][prof], h64["sigV"][prof]),
                "lambda": rel(h32["lambda_"][prof], h64["lambda_"][prof])},
            "fp64_retests": retests, "against": against}


def oracle_precision(lists, params, n_in: np.ndarray, args) -> dict:
    """FP32C and batched FP64 against the oracle (the reference's algorithm
    restated in C, all host threads) on the same haloes: the whole batch when
    it holds at most 6e7 entries, else its 20 longest lists plus a seeded
    random choice of ~2e7 entries of the others."""
    import torch
    from ahf_gb300 import lib, synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle as O
    from compare import compare, compare_fp32c
    O.build(ref=False)
    N = int(n_in.sum())
    if N <= 6e7:
        sel, what = np.arange(len(n_in)), "every halo of the batch"
    else:
        sel = synth.parity_halos(n_in, largest=20, sample_particles=2e7, seed=31)
        what = "the 20 longest lists and a seeded random choice of ~2e7 entries of the others"
    sub = lists.select(sel)
    t = {k: getattr(sub, k) for k in ("x", "y", "z", "vx", "vy", "vz", "w", "gidx")}
    t["off"] = torch.as_tensor(sub.off.astype(np.int64)).cuda()
    for k in ("cx", "cy", "cz"):
        t[k] = torch.as_tensor(getattr(sub, k)).cuda()
    db = lib.device_batch(t)   # raw pointers into `t`, which stays alive below
    r = lib.construct_halos_device(params, db, "batched_fp32c")
    retests = int(r.stats.n_retest)
    r32 = lib.fetch_result()
    lib.construct_halos_device(params, db, "batched_fp64")
    r64 = lib.fetch_result()
    host = sub.to_numpy()
    del db, t, sub
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    exp = O.run_oracle(params, host, 0)
    odt = time.perf_counter() - t0
    out = precision_report(r32, exp, retests, "the oracle (FP64, the reference's operation order) on " + what)
    out["batched_fp64_vs_oracle"] = {"kept_lists_identical": bool(np.array_equal(r64.member_off, exp.member_off)
                                                                   and np.array_equal(r64.member, exp.member)),
                                     "failures_at_1e-10": compare(r64, exp, rtol=1e-10, etol=1e-8)[:5]}
    out["fp32c_failures_at_bar"] = compare_fp32c(r32, exp)[:5]
    out["longest_list"] = int(n_in[sel].max())
    out["oracle_s"] = round(odt, 2)
    return out


def writer_leg(lists, res, args, ws: int, rank: int) -> dict:
    """The AHF_particles file of the last result on the GPU (ids = entry
    index, haloes by decreasing kept count), timed like the stage; the
    restated writer (snprintf per line, as the reference's fprintf) on a
    bounded sample of the haloes on one host core beside it."""
    import torch
    from ahf_gb300 import lib
    N = int(lists.x.numel())
    ids = torch.arange(N, dtype=torch.int64, device="cuda")
    npk = res.halo["npart"].astype(np.int64)
    order_np = np.argsort(-npk, kind="stable").astype(np.int64)
    order = torch.as_tensor(order_np).cuda()
    for _ in range(max(1, args.warmup)):
        addr, nb = lib.write_particles_device(ids, lists.w, order, 20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        addr, nb = lib.write_particles_device(ids, lists.w, order, 20)
    torch.cuda.synchronize()
    dt = allmax(ws, (time.perf_counter() - t0) / args.steps)
    lines = int(npk[npk >= 20].sum() + (npk >= 20).sum() + 1)
    out = {"metric": "AHF_particles bytes/s", "value": nb / dt, "unit": "bytes/s", "ms_per_step": dt * 1e3,
           "bytes": int(nb), "lines": lines, "lines_per_s": lines / dt, "cpu_baseline": None}
    # AHF_particles_bin (the AHFbinary build's file): 12 B per kept particle
    for _ in range(max(1, args.warmup)):
        addr, nbb = lib.write_particles_bin_device(ids, order, 20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        addr, nbb = lib.write_particles_bin_device(ids, order, 20)
    torch.cuda.synchronize()
    dtb = allmax(ws, (time.perf_counter() - t0) / args.steps)
    kept = int(npk[npk >= 20].sum())
    # algorithmic bytes: the kept entry (8 B) and its id (8 B) read, 12 B written
    alg = 28 * kept + 16 * int((npk >= 20).sum()) + 16
    out["binary"] = {"metric": "AHF_particles_bin bytes/s", "value": nbb / dtb, "unit": "bytes/s",
                     "ms_per_step": dtb * 1e3, "bytes": int(nbb), "particles": kept,
                     "algorithmic_bytes": alg, "achieved_gbs": alg / dtb / 1e9, "cpu_baseline": None}
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build(ref=False)
        sel = np.random.default_rng(29).permutation(len(npk))
        cum = np.cumsum(npk[sel])
        sel = np.sort(sel[:int(np.searchsorted(cum, 1e7)) + 1])
        moff = np.zeros(len(sel) + 1, np.uint64)
        moff[1:] = np.cumsum(npk[sel])
        mem = np.concatenate([res.member[int(res.member_off[h]):int(res.member_off[h + 1])] for h in sel])
        sub_order = np.argsort(-npk[sel], kind="stable").astype(np.int64)
        wn = lists.w.cpu().numpy() if lists.w is not None else None
        t1 = time.perf_counter()
        data = O.write_particles_oracle(np.arange(N, dtype=np.uint64), wn, moff, mem, npk[sel].astype(np.uint64),
                                        sub_order, 20)
        cdt = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": len(data) / cdt, "unit": "bytes/s", "cores": 1, "kind": "port",
                               "sample": f"the kept lists of {len(sel)} seeded random haloes ({len(data)} bytes), "
                                         f"snprintf per line, {cdt:.2f} s"}
        t1 = time.perf_counter()
        data = O.write_particles_bin_oracle(np.arange(N, dtype=np.uint64), moff, mem, npk[sel].astype(np.uint64),
                                            sub_order, 20)
        cdt = time.perf_counter() - t1
        out["binary"]["cpu_baseline"] = {"value": len(data) / cdt, "unit": "bytes/s", "cores": 1, "kind": "port",
                                         "sample": f"the same {len(sel)} haloes ({len(data)} bytes), a copy per "
                                                   f"field as the reference's fwrite calls, {cdt:.2f} s"}
    return out


def sfc_leg(lists, args, ws: int, rank: int) -> dict:
    """Hilbert keys and the particle order by key for the workload's
    particles as one snapshot (the keying loop and qsort of main.c:342-356),
    timed like the other legs; the restated keying and sort (C, one host
    core) on a bounded sample beside it."""
    import torch
    from ahf_gb300 import lib
    try:
        n = int(lists.x.numel())
        for _ in range(max(1, args.warmup)):
            keys, order = lib.sfc_sort_device(lists.x, lists.y, lists.z)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            keys, order = lib.sfc_sort_device(lists.x, lists.y, lists.z)
        torch.cuda.synchronize()
        dt = allmax(ws, (time.perf_counter() - t0) / args.steps)
        ok = bool((keys[1:] >= keys[:-1]).all().item())
        del keys, order
        torch.cuda.empty_cache()
        # algorithmic bytes: positions read (12 B), keys and order written (16 B)
        out = {"metric": "particles keyed and sorted/s", "value": n / dt, "unit": "particles/s",
               "ms_per_step": dt * 1e3, "n_particles": n, "keys_ascending": ok,
               "algorithmic_bytes": 28 * n, "achieved_gbs": 28 * n / dt / 1e9, "cpu_baseline": None}
        if rank == 0 and not args.no_cpu:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as O
            O.build(ref=False)
            m = min(n, 5_000_000)
            xs = [v[:m].cpu().numpy() for v in (lists.x, lists.y, lists.z)]
            t1 = time.perf_counter()
            O.sfc_sort_oracle(*xs)
            cdt = time.perf_counter() - t1
            out["cpu_baseline"] = {"value": m / cdt, "unit": "particles/s", "cores": 1, "kind": "port",
                                   "sample": f"the first {m} particles, keys and qsort, {cdt:.2f} s"}
    except Exception as e:   # noqa: BLE001 -- reported in the line, the other legs stand
        return {"error": str(e)[:300]}
    return out


def amr_leg(args, rank: int) -> dict:
    """AHF's AMR hierarchy on the GPU for the cfg1 and cfg2 boxes (64^3 and
    256^3 particles; LgridDomain 64, LgridMax 16384, NperDomCell =
    NperRefCell = 5): the domain grid and every refinement with its relink
    and TSC densities (ahfgpu_amr_hierarchy_device), timed with CUDA events
    over W warm-up and K timed calls; beside it the reference's own
    gen_domgrids + ll + assign_npart + gen_AMRhierarchy (compiled from its
    sources, libamr_serial: one host core, timed inside a child process
    around the call) on the same particles, with its grid counts checked
    against the GPU's."""
    import torch
    from ahf_gb300 import lib, synth
    out = {}
    try:
        for name in ("cfg1", "cfg2"):
            S = synth.box_snapshot(name)
            p = (S.pos / np.float32(S.box)).astype(np.float32)
            x, y, z = (torch.as_tensor(np.ascontiguousarray(p[:, k])).cuda() for k in range(3))
            n = len(S.ids)
            for _ in range(max(1, args.warmup)):
                lv = lib.amr_hierarchy_device(x, y, z, 64, 16384, 5.0, 5.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                lv = lib.amr_hierarchy_device(x, y, z, 64, 16384, 5.0, 5.0)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            leg = {"metric": "particles through the AMR hierarchy/s", "value": n / (ms / 1e3),
                   "unit": "particles/s", "ms_per_step": ms, "n_particles": n, "ngrid_dom": 64,
                   "grids": lv.tolist(), "timing": "CUDA events around the call (it synchronises per level)",
                   "cpu_baseline": None}
            if rank == 0 and not args.no_cpu:
                sys.path.insert(0, os.path.join(ROOT, "oracle"))
                import oracle as O
                O.build()
                if os.path.isfile(O.ref_amr_path()):
                    ref, sec = O.amr_levels_reference(p[:, 0], p[:, 1], p[:, 2], 64, 16384, 5.0, 5.0, timed=True)
                    leg["cpu_baseline"] = {"value": n / sec, "unit": "particles/s", "cores": 1, "kind": "reference",
                                           "sample": f"the whole box, gen_domgrids + ll + assign_npart + "
                                                     f"gen_AMRhierarchy, {sec:.3f} s",
                                           "same_grids": bool(np.array_equal(ref, lv))}
            out[name] = leg
            del x, y, z
    except Exception as e:   # noqa: BLE001 -- reported in the line, the other legs stand
        out["error"] = str(e)[:300]
    return out


def gather_radii(lists, n_in: np.ndarray):
    """Per halo: the farthest periodic distance of its own list's particles
    from its centre (the lists were drawn out to 1.5 R_vir), on the GPU."""
    import torch
    dev = lists.x.device
    hid = torch.repeat_interleave(torch.arange(len(n_in), device=dev), torch.as_tensor(n_in, device=dev))
    d2 = torch.zeros(len(hid), dtype=torch.float64, device=dev)
    for a, c in ((lists.x, lists.cx), (lists.y, lists.cy), (lists.z, lists.cz)):
        d = (a.double() - torch.as_tensor(c, device=dev)[hid]).abs()
        d = torch.where(d > 0.5, 1.0 - d, d)
        d2 += d * d
        del d
    m = torch.zeros(len(n_in), dtype=torch.float64, device=dev).scatter_reduce(0, hid, d2, "amax")
    return m.sqrt()


def gather_leg(lists, n_in: np.ndarray, args, ws: int, rank: int) -> dict:
    """The particle gather (ahfgpu_gather_device) on the workload's lists as
    one snapshot: every list particle once, each halo's radius the farthest
    of its own particles.  Timed like the stage (CUDA events, W warm-up
    calls), with the restated gather's grid search on a bounded sample of the
    haloes on the host cores beside it."""
    import torch
    from ahf_gb300 import lib
    parts = {k: getattr(lists, k) for k in ("x", "y", "z", "vx", "vy", "vz", "w")}
    rad = gather_radii(lists, n_in)
    cen = {"cx": torch.as_tensor(lists.cx).cuda(), "cy": torch.as_tensor(lists.cy).cuda(),
           "cz": torch.as_tensor(lists.cz).cuda(), "rad": rad}
    torch.cuda.synchronize()
    for _ in range(max(1, args.warmup)):
        b = lib.gather_device(parts, cen)
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b = lib.gather_device(parts, cen)
    torch.cuda.synchronize()
    dt = allmax(ws, (time.perf_counter() - t0) / args.steps)
    off, _ = lib.gathered_lists(b)
    ng = int(off[-1])
    out = {"metric": "particles gathered/s", "value": allsum(ws, float(ng)) / dt, "unit": "particles/s",
           "ms_per_step": dt * 1e3, "n_particles": int(lists.x.numel()), "n_halos": int(len(n_in)),
           "n_gathered": ng, "workload": f"{args.workload} lists as one snapshot, radius = farthest own particle",
           "timing": "host wall clock around each synchronous call", "cpu_baseline": None}
    # gather radii (spatialRef2halos' loop): every halo against every halo
    # with more particles; R_vir stands in as 2/3 of the list radius, the cap
    # is AHF's default MaxGatherRad = 3 Mpc/h over the box
    npart = torch.as_tensor(n_in.astype(np.int64)).cuda()
    rvir = rad / 1.5
    maxg = 3.0 / float(lists.boxsize)
    for _ in range(max(1, args.warmup)):
        gr = lib.gather_radii_device(npart, cen["cx"], cen["cy"], cen["cz"], rvir, maxg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gr = lib.gather_radii_device(npart, cen["cx"], cen["cy"], cen["cz"], rvir, maxg)
    torch.cuda.synchronize()
    rdt = (time.perf_counter() - t0) / args.steps

    def pairs(counts):
        srt = np.sort(counts)
        return float(np.sum(len(srt) - np.searchsorted(srt, counts, side="right")))
    npairs = pairs(n_in)
    out["radii"] = {"metric": "halo pairs/s", "value": npairs / rdt, "unit": "pairs/s", "ms_per_step": rdt * 1e3,
                    "n_halos": int(len(n_in)), "n_pairs": npairs, "cpu_baseline": None}
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build(ref=False)
        rs = np.random.default_rng(23).choice(len(n_in), size=min(len(n_in), 20000), replace=False)
        cxyz = [np.asarray(getattr(lists, k))[rs] for k in ("cx", "cy", "cz")]
        t1 = time.perf_counter()
        O.gather_radii_oracle(n_in[rs].astype(np.uint64), cxyz[0], cxyz[1], cxyz[2], rvir.cpu().numpy()[rs], maxg)
        rcdt = time.perf_counter() - t1
        out["radii"]["cpu_baseline"] = {"value": pairs(n_in[rs]) / rcdt, "unit": "pairs/s", "cores": os.cpu_count() or 1,
                                        "kind": "port", "sample": f"{len(rs)} seeded random haloes as their own "
                                                                  f"catalogue, {rcdt:.2f} s"}
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build(ref=False)
        samp = cpu_sample(n_in, args.gather_cpu_particles, seed=17)
        sub = _device_subset(lists, samp)
        xs = {k: sub[k].cpu().numpy() for k in ("x", "y", "z")}
        r = rad[torch.as_tensor(samp, device=rad.device)].cpu().numpy()
        c = [np.asarray(getattr(lists, k))[samp] for k in ("cx", "cy", "cz")]
        t1 = time.perf_counter()
        coff, _ = O.gather_oracle(xs["x"], xs["y"], xs["z"], c[0], c[1], c[2], r)
        cdt = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": float(coff[-1]) / cdt, "unit": "particles/s", "cores": os.cpu_count() or 1,
                               "kind": "port",
                               "sample": f"the lists of {len(samp)} seeded random haloes ({int(coff[-1])} gathered) "
                                         f"as their own snapshot, grid search, {cdt:.2f} s"}
    return out


def cpu_sample(n_in: np.ndarray, target: float, seed: int = 99) -> np.ndarray:
    """Deterministic random subset of haloes with about `target` particles,
    drawn so the size mix follows the full batch."""
    rng = np.random.default_rng(seed)
    order = rng.permutation(len(n_in))
    cs = np.cumsum(n_in[order])
    k = int(np.searchsorted(cs, target)) + 1
    return np.sort(order[:max(1, min(k, len(order)))])


def _device_subset(lists, halos):
    """torch dict of a halo subset of a device-resident HaloLists."""
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


def host_lists(lists):
    """numpy copy of a torch-resident HaloLists."""
    return lists.to_numpy()


def run_cpu(params, lists_np, sample, nthreads, keep_order: bool = False):
    """One CPU run over the haloes `sample` (ascending, unless keep_order)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    sub = lists_np.select(sample if keep_order else np.sort(sample))
    kind = "port"
    fn = O.run_oracle
    if O.have_ref(sub.w is not None):
        kind, fn = "reference", O.run_reference
    t0 = time.perf_counter()
    fn(params, sub, nthreads)
    dt = time.perf_counter() - t0
    return sub.n, dt, kind


# ---------------------------------------------------------------- arms

def workload_config(args, n_in: np.ndarray, ws: int) -> dict:
    """The `config` of both arms' lines (the same dict for the same workload)."""
    N = int(n_in.sum())
    desc = {"cfg1": "cfg1: 20 NFW haloes of 25-2,500 particles in 50 Mpc/h, lists to 1.5 R_vir",
            "cfg2": "cfg2: 2,000 haloes, N_p ~ N^-1.9 on [20,1e6], 3 subhaloes per host above 1e4",
            "cfg3": "cfg3: 1e5 halo particle lists, N_p ~ N^-1.56 on [20,2e6], float32 pos/vel, 64-bit ids",
            "cfg4": "cfg4: 40,000 NFW haloes of 25-2,500 particles in 400 Mpc/h, lists to 1.5 R_vir",
            "cfg5": "cfg5: 5e5 haloes, N_p ~ N^-1.9 on [20,1e6], 3 subhaloes per host above 1e4"}
    return {"workload": desc.get(args.workload, args.workload) +
            (", two species 5:1 (15% heavy)" if args.multimass else ", equal masses"),
            "n_halos": int(len(n_in)), "n_particles": N, "scale": args.scale, "multimass": bool(args.multimass),
            "l2": "inputs (%.1f GB) larger than L2 (129 MB): no flush" % (N * 32 / 1e9),
            "parallelism": f"{ws} rank(s); the batch's haloes split over the ranks (LPT on n log n), "
                           f"no data-path collective"}


def reference_arm(args, ws, rank):
    """The reference's own routines (compiled from its sources; the C
    restatement where they could not be built) on all host threads.  The K
    timed steps together process the whole workload once: halo i of the
    batch sorted by decreasing list length goes to step i mod K, and each
    step runs its haloes largest first under OpenMP's dynamic schedule, as
    the reference's loop does.  Warm-up steps run small seeded samples."""
    if rank != 0:
        return
    import torch
    from ahf_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=None)
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    lists = synth.generate(args.workload, scale=args.scale, device=dev, multimass=args.multimass, as_numpy=True)
    params = synth.params_for(lists)
    n_in = np.diff(lists.off.astype(np.int64))
    nthreads = os.cpu_count() or 1
    order = np.argsort(-n_in, kind="stable")
    K = max(1, args.steps)
    for s in range(args.warmup):
        run_cpu(params, lists, cpu_sample(n_in, min(2e6, float(n_in.sum())), seed=1000 + s), nthreads)
    times, parts, kind = [], [], "port"
    for k in range(K):
        n, dt, kind = run_cpu(params, lists, order[k::K], nthreads, keep_order=True)
        times.append(dt)
        parts.append(n)
    value = float(np.sum(parts) / np.sum(times))
    serial = None
    if args.cpu_serial_particles > 0:
        samp1 = cpu_sample(n_in, args.cpu_serial_particles, seed=23)
        n1, dt1, kind1 = run_cpu(params, lists, samp1, 1)
        serial = {"value": n1 / dt1, "unit": UNIT, "cores": 1, "kind": kind1,
                  "sample": f"seeded random subset of {len(samp1)} haloes / {n1} particles, one thread, {dt1:.2f} s"}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, n_in, args.gpus),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind,
                         "sample": f"the whole workload ({int(np.sum(parts))} particles) over the {K} timed steps: "
                                   f"haloes dealt round-robin by decreasing length, {nthreads} OpenMP threads, "
                                   f"{np.sum(times):.1f} s in all",
                         "serial": serial},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ours_arm(args, ws, rank, local):
    import ctypes as C

    import torch
    from ahf_gb300 import abi, lib, synth
    from ahf_gb300 import build as B

    B.build()
    torch.cuda.set_device(local)
    lib.init(local)
    mode = args.mode or "batched_fp32c"
    # every rank builds the same seeded batch and keeps its share of the
    # haloes (the library's LPT split, ahfgpu_shard_halos)
    lists = synth.generate(args.workload, scale=args.scale, device="cuda", multimass=args.multimass,
                           as_numpy=False)
    params = synth.params_for(lists)
    n_full = np.diff(lists.off.astype(np.int64))
    if ws > 1:
        from ahf_gb300.shard import lpt_assign
        mine = np.nonzero(lpt_assign(n_full, ws) == rank)[0]
        lists = lists.select(mine)
        torch.cuda.empty_cache()
    n_in = np.diff(lists.off.astype(np.int64))
    N = int(n_in.sum())
    t = {"off": torch.as_tensor(lists.off.astype(np.int64)).cuda()}
    for k in ("x", "y", "z", "vx", "vy", "vz", "w"):
        t[k] = getattr(lists, k)
    t["gidx"] = lists.gidx
    for k in ("cx", "cy", "cz"):
        t[k] = torch.as_tensor(getattr(lists, k)).cuda()
    # page-locked host copies of the inputs for the e2e leg, made first as a
    # caller's particle arrays would be (they exist before the stage runs,
    # written by the host: AHF reads them from the snapshot files)
    host = {}
    if not args.no_e2e:
        for k in ("x", "y", "z", "vx", "vy", "vz", "w", "gidx"):
            v = getattr(lists, k)
            if v is None:
                host[k] = None
                continue
            hp = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
            hp.copy_(v.cpu())   # through pageable memory: the host writes the pinned pages
            host[k] = hp
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    db = lib.device_batch(t)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def step(m):
        r = lib.construct_halos_device(params, db, m, sh)
        return r

    # warm-up
    for _ in range(args.warmup):
        r = step(mode)
    barrier(ws)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kern_ms, launches = [], 0
    e0.record(stream)
    for _ in range(args.steps):
        r = step(mode)
        kern_ms.append(r.stats.ms_device)
        launches += r.stats.n_launches
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    barrier(ws)
    ms = e0.elapsed_time(e1) / args.steps
    ms_max = allmax(ws, ms)
    total_parts = allsum(ws, float(N))
    value = total_parts / (ms_max / 1e3)
    res = lib.fetch_result()
    stats = r.stats
    # e2e through the host API with pinned buffers, right after the
    # device-resident loop: measured after the other forms and their host-side
    # result checks instead, the same calls took 490-590 ms (slower input and
    # result copies) against 465 ms here
    e2e = None
    if not args.no_e2e:
        hb = abi.Batch()
        off_np = np.ascontiguousarray(lists.off.astype(np.uint64))
        cen = {k: np.ascontiguousarray(getattr(lists, k)) for k in ("cx", "cy", "cz")}
        hb.nhalo = len(n_in)
        hb.off = off_np.ctypes.data_as(C.POINTER(C.c_uint64))
        for k in ("x", "y", "z", "vx", "vy", "vz", "w"):
            setattr(hb, k, C.cast(C.c_void_p(host[k].data_ptr() if host[k] is not None else None),
                                  C.POINTER(C.c_float)))
        hb.gidx = C.cast(C.c_void_p(host["gidx"].data_ptr()), C.POINTER(C.c_uint64))
        for k in ("cx", "cy", "cz"):
            setattr(hb, k, cen[k].ctypes.data_as(C.POINTER(C.c_double)))
        torch.cuda.synchronize()
        for _ in range(max(1, min(args.warmup, 2))):
            rr = lib.construct_halos_raw(params, hb, mode)
            lib.free_result(rr)
        barrier(ws)
        e2e_steps = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        d2h = 0
        lib_total, lib_dev, lib_parts = [], [], []
        for _ in range(e2e_steps):
            rr = lib.construct_halos_raw(params, hb, mode)
            nk = rr.stats.n_kept
            d2h = nk * 8 + len(n_in) * (C.sizeof(abi.Halo) + 16) + 8 * 25 * int(res.prof_off[-1])
            lib_total.append(rr.stats.ms_total)
            lib_dev.append(rr.stats.ms_device)
            lib_parts.append([getattr(rr.stats, k) for k in ("ms_plan", "ms_h2d", "ms_h2d_first", "ms_pack", "ms_d2h")])
            lib.free_result(rr)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / e2e_steps
        dt = allmax(ws, dt)
        h2d = N * (24 + (4 if lists.w is not None else 0) + 8) + len(n_in) * 32
        e2e = {"value": total_parts / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": dt * 1e3, "ms_in_library": float(np.mean(lib_total)),
               "ms_device": float(np.mean(lib_dev))}
        for k, v in zip(("ms_plan", "ms_h2d", "ms_h2d_first", "ms_pack", "ms_d2h"), np.mean(lib_parts, axis=0)):
            e2e[k] = float(v)
        e2e["ms_per_call"] = [round(float(v), 2) for v in lib_total]
        e2e["host_buffers"] = "page-locked (torch pin_memory)"
        # the same call from pageable host arrays, as a C caller's malloc'd
        # arrays are: the input copies then go through the driver's staging
        pg = {k: (np.ascontiguousarray(host[k].numpy()).copy() if host[k] is not None else None)
              for k in ("x", "y", "z", "vx", "vy", "vz", "w", "gidx")}
        hp = abi.Batch()
        hp.nhalo, hp.off = hb.nhalo, hb.off
        for k in ("x", "y", "z", "vx", "vy", "vz", "w"):
            setattr(hp, k, C.cast(C.c_void_p(pg[k].ctypes.data if pg[k] is not None else None),
                                  C.POINTER(C.c_float)))
        hp.gidx = C.cast(C.c_void_p(pg["gidx"].ctypes.data), C.POINTER(C.c_uint64))
        for k in ("cx", "cy", "cz"):
            setattr(hp, k, getattr(hb, k))
        rr = lib.construct_halos_raw(params, hp, mode)
        lib.free_result(rr)
        barrier(ws)
        t0 = time.perf_counter()
        pg_parts = []
        for _ in range(e2e_steps):
            rr = lib.construct_halos_raw(params, hp, mode)
            pg_parts.append([rr.stats.ms_total, rr.stats.ms_h2d, rr.stats.ms_device])
            lib.free_result(rr)
        pdt = allmax(ws, (time.perf_counter() - t0) / e2e_steps)
        m = np.mean(pg_parts, axis=0)
        e2e["pageable"] = {"value": total_parts / pdt, "unit": UNIT, "ms_per_step": pdt * 1e3,
                           "ms_in_library": float(m[0]), "ms_h2d": float(m[1]), "ms_device": float(m[2]),
                           "host_buffers": "pageable (numpy arrays)"}
        del pg
    tuning = {k: v for k, v in lib.tuning(local).items() if k in ("class_max", "class_bps", "source")}
    if tuning.get("source", "").endswith(".json"):
        tuning["source"] = os.path.basename(tuning["source"])
    headline_stats = {"replay_halos": int(stats.n_replay_halos), "key_ties": int(stats.n_key_ties),
                      "retests": int(stats.n_retest), "fp64_halos": int(stats.n_fp64_halos)}
    balg = alg_bytes(n_in, res.halo, lists.w is not None)
    kms = float(np.mean(kern_ms))
    hbm, peak_kind = peaks()
    achieved = balg / (kms / 1e3) / 1e9
    kname = "halo_fp64_kernel" if "fp64" in mode else "halo_fp32c_kernel"
    tpp = ncu_traffic(args.workload, kname)
    traffic = tpp * N if tpp is not None else None

    # the AHF_particles bytes of this result (ahfgpu_write_particles_device)
    writer = None
    if not args.no_writer:
        writer = writer_leg(lists, res, args, ws, rank)

    # other forms, once each (same workload)
    forms = {}
    precision = None
    if args.forms != "none":
        want = ["batched_fp32c", "batched_fp64", "plain_fp64"] if args.forms == "all" else args.forms.split(",")
        for f in want:
            if f == mode:
                forms[f] = {"value": value, "ms_per_step": ms, "sample": "whole workload"}
                continue
            try:
                db_f, nf, desc = db, N, "whole workload"
                if f == "plain_fp64":
                    # one launch per halo: timed on a bounded random sample of the haloes
                    samp = cpu_sample(n_in, args.plain_particles, seed=7)
                    sub = _device_subset(lists, samp)
                    db_f, nf = lib.device_batch(sub), int(n_in[samp].sum())
                    desc = f"seeded random subset of {len(samp)} haloes / {nf} particles"
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                lib.construct_halos_device(params, db_f, f, sh)
                a.record(stream)
                rr = lib.construct_halos_device(params, db_f, f, sh)
                b.record(stream)
                torch.cuda.synchronize()
                fms = a.elapsed_time(b)
                forms[f] = {"value": nf / (fms / 1e3), "ms_per_step": fms, "sample": desc,
                            "replay_halos": int(rr.stats.n_replay_halos)}
                if f == "batched_fp64" and mode == "batched_fp32c":
                    precision = {"vs_fp64": precision_report(
                        res, lib.fetch_result(), int(stats.n_retest),
                        "the batched FP64 form (bit-exact to the reference) on the whole batch")}
            except lib.AhfGpuError as e:
                forms[f] = {"unavailable": str(e)}
        if mode == "batched_fp32c" and rank == 0 and not args.no_cpu:
            try:
                precision = dict(precision or {})
                precision["vs_oracle"] = oracle_precision(lists, params, n_in, args)
            except Exception as e:   # noqa: BLE001 -- reported in the line, the other legs stand
                precision["vs_oracle"] = {"error": str(e)[:300]}
        # leave the last result of the headline form in place for fetch_result()
        step(mode)
        torch.cuda.synchronize()


    gather = None
    if not args.no_gather:
        gather = gather_leg(lists, n_in, args, ws, rank)

    cpu = None
    if rank == 0 and not args.no_cpu:
        lists_np = host_lists(lists)
        samp = cpu_sample(n_in, args.cpu_particles)
        nthreads = os.cpu_count() or 1
        runs = [run_cpu(params, lists_np, samp, nthreads) for _ in range(max(1, args.cpu_repeats))]
        n, dt, kind = min(runs, key=lambda r: r[1])
        cpu = {"value": n / dt, "unit": UNIT, "cores": nthreads, "kind": kind,
               "sample": f"seeded random subset of {len(samp)} haloes / {n} particles of the workload, "
                         f"{nthreads} OpenMP threads, best of {len(runs)}: {dt:.2f} s"}
        if args.cpu_serial_particles > 0:
            # the serial build's rate (one host core), beside the threaded one
            samp1 = cpu_sample(n_in, args.cpu_serial_particles, seed=23)
            n1, dt1, kind1 = run_cpu(params, lists_np, samp1, 1)
            cpu["serial"] = {"value": n1 / dt1, "unit": UNIT, "cores": 1, "kind": kind1,
                             "sample": f"seeded random subset of {len(samp1)} haloes / {n1} particles, "
                                       f"one thread, {dt1:.2f} s"}
    # the Hilbert keying and particle sort (ahfgpu_sfc_sort_device), last:
    # a failure here is reported in its key and costs no other number
    sfc = None if args.no_sfc else sfc_leg(lists, args, ws, rank)
    amr = None if args.no_amr else amr_leg(args, rank)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64" if "fp64" in mode else "f32+f64", "data": "synthetic",
        "config": workload_config(args, n_full, ws),
        "run": {"form": mode, "n_kept": int(stats.n_kept), "tuning": tuning},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": kname,
                     "alg_bytes_per_launch": balg, "kernel_ms": kms},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": ck,
        "gpu_launches": int(launches),
        "forms": forms,
        "gather": gather,
        "writer": writer,
        "sfc_sort": sfc,
        "amr": amr,
        "precision": precision,
        "diagnostics": headline_stats,
    }
    print(json.dumps(line), flush=True)


PHASE_NAMES = {0: "keys", 1: "sort", 2: "near ties + gather", 3: "R_vir cut + first potential", 4: "unbinding",
               5: "second R_vir cut", 6: "profiles", 7: "kept lists",
               10: "  unbinding: tile loads", 11: "  unbinding: bound fixpoint", 12: "  unbinding: potential + writes",
               16: "  profiles: ranks", 17: "  profiles: bins", 18: "  profiles: loads", 19: "  profiles: terms",
               20: "  profiles: scans", 21: "  profiles: most bound", 22: "  profiles: bin rows",
               25: "  profiles: find_max", 27: "    find_max: FP64 re-check", 30: "    find_max: FP32 screen"}


def phase_case() -> None:
    """Per-phase SM cycles per list entry (summed over the CTAs of the second
    of two calls) of the FP32C stage on the class-2 lists of the seeded
    1e5-halo batch, from an instrumented build of the library (slots
    kPhaseSlots of ahfgpu_debug_phase: 0-7 the phases, 10-30 sub-phases)."""
    import ctypes as C
    from ahf_gb300 import build as B
    out = os.path.join(ROOT, "ahf_gb300", "_build", "libahfgpu_phases.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    B.build(defines=("AHFGPU_PHASE_TIMERS",), out=out)
    os.environ["AHFGPU_LIB"] = out
    from ahf_gb300 import lib, synth   # the first import of lib in this process: it loads `out`
    L = lib.load()
    L.ahfgpu_debug_phase.argtypes = [C.c_void_p, C.c_int]
    L.ahfgpu_debug_phase.restype = C.c_int
    lib.init(0)
    Lst = synth.generate("cfg3", device="cuda", as_numpy=False)
    n = np.diff(Lst.off.astype(np.int64))
    sel = np.nonzero(n > 32768)[0]
    t = _device_subset(Lst, sel)
    db = lib.device_batch(t)
    p = synth.params_for(Lst)
    ph = np.zeros(32, np.uint64)
    lib.construct_halos_device(p, db, "batched_fp32c")
    L.ahfgpu_debug_phase(ph.ctypes.data, 1)
    r = lib.construct_halos_device(p, db, "batched_fp32c")
    L.ahfgpu_debug_phase(ph.ctypes.data, 1)
    N = int(n[sel].sum())
    tot = float(sum(int(ph[k]) for k in range(8)))
    print(f"phases: {len(sel)} lists, {N} entries, {r.stats.ms_device:.2f} ms (instrumented), "
          f"{tot / N:.1f} SM cycles per entry")
    for k in sorted(PHASE_NAMES):
        if ph[k]:
            print(f"  {PHASE_NAMES[k]:36s} {float(ph[k]) / N:8.2f}")


def profile_case(args) -> None:
    """One small device-resident case, run twice, for a profiler: the stage on
    lists cut from the seeded 1e5-halo batch (small: 3000 lists of <= 512
    entries, medium: 300 of 2048-16384, big: the one nearest 2e5), the gather
    on the lists of 1e5 * scale haloes as a snapshot, or the Hilbert key sort
    of n seeded uniform points."""
    if args.case == "phases":
        phase_case()
        return
    import torch
    from ahf_gb300 import build as B
    from ahf_gb300 import lib, synth
    B.build()
    lib.init(0)
    mode = args.mode or "batched_fp32c"
    if args.case == "sfc":
        n = int(args.case_arg or 5e7)
        g = torch.Generator(device="cuda")
        g.manual_seed(5)
        x, y, z = (torch.rand(n, device="cuda", generator=g) for _ in range(3))
        ms = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            keys, _order = lib.sfc_sort_device(x, y, z)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        ok = bool((keys[1:] >= keys[:-1]).all().item())
        print(f"sfc: points {n} ascending {ok} ms per call {', '.join(f'{m:.2f}' for m in ms)}")
        return
    if args.case == "amr":
        S = synth.box_snapshot("cfg2")
        p = (S.pos / np.float32(S.box)).astype(np.float32)
        x, y, z = (torch.as_tensor(np.ascontiguousarray(p[:, k])).cuda() for k in range(3))
        ms = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            lv = lib.amr_hierarchy_device(x, y, z, 64, 16384, 5.0, 5.0)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        print(f"amr: particles {len(S.ids)} grids {lv.tolist()} "
              f"ms per call {', '.join(f'{m:.2f}' for m in ms)}")
        return
    scale = (args.case_arg or 0.05) if args.case == "gather" else 0.05
    L = synth.generate("cfg3", scale=0.15 if args.case == "large" else scale, device="cuda", as_numpy=False)
    n = np.diff(L.off.astype(np.int64))
    if args.case == "gather":
        rad = gather_radii(L, n)
        parts = {k: getattr(L, k) for k in ("x", "y", "z", "vx", "vy", "vz", "w")}
        cen = {"cx": torch.as_tensor(L.cx).cuda(), "cy": torch.as_tensor(L.cy).cuda(),
               "cz": torch.as_tensor(L.cz).cuda(), "rad": rad}
        ms = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b = lib.gather_device(parts, cen)
            ms.append((time.perf_counter() - t0) * 1e3)
        off, _ = lib.gathered_lists(b)
        print(f"gather: haloes {len(n)} particles {int(L.x.numel())} gathered {int(off[-1])} "
              f"ms per call {', '.join(f'{m:.1f}' for m in ms)}")
        return
    if args.case == "small":
        sel = np.nonzero(n <= 512)[0][:3000]
    elif args.case == "medium":
        sel = np.nonzero((n > 2048) & (n <= 16384))[0][:300]
    elif args.case == "large":
        sel = np.sort(np.argsort(np.abs(n - 100000), kind="stable")[:160])
    else:
        sel = np.array([int(np.argmin(np.abs(n - 200000)))])
    p = synth.params_for(L)
    t = _device_subset(L, sel)
    db = lib.device_batch(t)   # raw pointers into `t`, kept alive to the end
    for _ in range(2):
        r = lib.construct_halos_device(p, db, mode)
    res = lib.fetch_result()
    print(f"{args.case} {mode}: haloes {len(sel)} particles {int(n[sel].sum())} ms {r.stats.ms_device:.3f} "
          f"fix_rounds max {res.halo['fix_rounds'].max()} niter mean {res.halo['niter'].mean():.2f} "
          f"retests {r.stats.n_retest} exact_iterations {r.stats.n_replay_halos}")


def main():
    args = parse()
    if args.case:
        profile_case(args)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, ws, rank)
    else:
        ours_arm(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
