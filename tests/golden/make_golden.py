"""Regenerate the golden fixtures in this directory.

Runs the UNMODIFIED reference routines (oracle/_ref/libahfref*.so, built by
oracle/Makefile from the AHF source tree) on small seeded inputs and stores
inputs and outputs as .npz.  The reference has no test suite and ships no
data, so these fixtures are the pinned known answers for the restatement and
the GPU library.  Run from the repository root:

    python tests/golden/make_golden.py

Cases: a cfg1-like snapshot slice, a MULTIMASS two-species slice, subhalo
lists, and hand-built edge cases (empty list, fewer than MINPART particles,
haloes straddling the periodic boundary, a particle exactly at the centre,
every particle unbound, the innermost particle unbound, a halo that falls
below MINPART during unbinding, list sizes around warp/block boundaries).
The gather fixtures (gather_*.npz) hold the reference's own particle gather
(ahf_halos_sfc_gatherParts with its Hilbert-key setup) on a cfg1 snapshot and
on hand-built periodic-boundary and radius edge cases; writer_cfg1.npz the
reference's AHF_particles bytes for the cfg1 haloes.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ahf_gb300 import synth  # noqa: E402
from ahf_gb300.abi import Params  # noqa: E402
from ahf_gb300.synth import HaloLists  # noqa: E402

PARAM_FIELDS = [f[0] for f in Params._fields_]


def params_to_array(p) -> np.ndarray:
    return np.array([float(getattr(p, f)) for f in PARAM_FIELDS])


def params_from_array(a) -> Params:
    p = Params()
    for f, v in zip(PARAM_FIELDS, a):
        setattr(p, f, int(v) if f == "MINPART" else float(v))
    return p


def save_case(name: str, params, lists: HaloLists, res) -> None:
    d = dict(params=params_to_array(params), off=lists.off, x=lists.x, y=lists.y, z=lists.z,
             vx=lists.vx, vy=lists.vy, vz=lists.vz, gidx=lists.gidx, cx=lists.cx, cy=lists.cy,
             cz=lists.cz, out_member_off=res.member_off, out_member=res.member,
             out_prof_off=res.prof_off, out_prof=res.prof)
    if lists.w is not None:
        d["w"] = lists.w
    for f in res.halo.dtype.names:
        d["out_halo_" + f] = res.halo[f]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)


def load_case(path: str):
    """(params, HaloLists, expected dict) from a fixture file."""
    z = np.load(path)
    w = z["w"] if "w" in z.files else None
    lists = HaloLists(z["off"], z["x"], z["y"], z["z"], z["vx"], z["vy"], z["vz"], w, z["gidx"],
                      z["cx"], z["cy"], z["cz"], 0.0, 0.0, os.path.basename(path))
    exp = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return params_from_array(z["params"]), lists, exp


def concat(parts: list[HaloLists]) -> HaloLists:
    off = [np.zeros(1, np.uint64)]
    base = 0
    for p in parts:
        off.append(p.off[1:] + np.uint64(base))
        base += p.n
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])
    w = None if parts[0].w is None else cat("w")
    return HaloLists(np.concatenate(off), cat("x"), cat("y"), cat("z"), cat("vx"), cat("vy"), cat("vz"), w,
                     np.arange(base, dtype=np.uint64), cat("cx"), cat("cy"), cat("cz"),
                     parts[0].boxsize, parts[0].pmass, "concat")


def edge_cases(base: HaloLists) -> HaloLists:
    """Hand-built lists from the haloes of `base` (each one a copy of a
    cfg1-like halo, modified)."""
    rng = np.random.default_rng(777)
    parts = []
    sizes = np.diff(base.off).astype(np.int64)
    big = int(np.argmax(sizes))

    def one(h, n=None):
        s = base.select([h])
        if n is not None:
            s = trim(s, n)
        return s

    def trim(s, n):
        keep = np.arange(min(n, s.n))
        off = np.array([0, len(keep)], np.uint64)
        return HaloLists(off, s.x[keep], s.y[keep], s.z[keep], s.vx[keep], s.vy[keep], s.vz[keep],
                         None if s.w is None else s.w[keep], s.gidx[keep], s.cx, s.cy, s.cz,
                         s.boxsize, s.pmass)

    # empty list and a list below MINPART
    e = one(big, 0)
    parts.append(e)
    parts.append(one(big, 7))
    # straddling the periodic boundary: move the halo's centre to the corner
    for corner in ([0.0005, 0.9995, 0.5], [0.9999, 0.0001, 0.00005]):
        s = one(big)
        shift = np.array(corner) - np.array([s.cx[0], s.cy[0], s.cz[0]])
        for k, ck in zip(("x", "y", "z"), ("cx", "cy", "cz")):
            i = "xyz".index(k)
            v = np.mod(getattr(s, k).astype(np.float64) + shift[i], 1.0).astype(np.float32)
            v[v >= 1.0] = 0.0
            setattr(s, k, v)
            setattr(s, ck, np.mod(getattr(s, ck) + shift[i], 1.0))
        parts.append(s)
    # a particle exactly at the centre (distance 0 -> the MACHINE_ZERO branch)
    s = one(big)
    s.cx = s.x[3:4].astype(np.float64).copy()
    s.cy = s.y[3:4].astype(np.float64).copy()
    s.cz = s.z[3:4].astype(np.float64).copy()
    parts.append(s)
    s = one(big)
    for k, ck in zip(("x", "y", "z"), ("cx", "cy", "cz")):
        a = getattr(s, k).copy()
        a[5] = np.float32(getattr(s, ck)[0])
        setattr(s, k, a)
        setattr(s, ck, a[5:6].astype(np.float64))
    parts.append(s)
    # every particle unbound: huge velocities
    s = one(big)
    s.vx = (s.vx * 1e4).astype(np.float32)
    s.vy = (s.vy * 1e4).astype(np.float32)
    s.vz = (s.vz * 1e4).astype(np.float32)
    parts.append(s)
    # innermost particles unbound: boost the 12 nearest
    s = one(big)
    d2 = (s.x - s.cx[0]) ** 2 + (s.y - s.cy[0]) ** 2 + (s.z - s.cz[0]) ** 2
    near = np.argsort(d2)[:12]
    for k in ("vx", "vy", "vz"):
        a = getattr(s, k).copy()
        a[near] = a[near] * 200.0
        setattr(s, k, a)
    parts.append(s)
    # falls below MINPART during unbinding: small halo, most particles fast
    s = one(int(np.argmin(np.where(sizes >= 30, sizes, 1 << 30))))
    fast = rng.random(s.n) < 0.6
    for k in ("vx", "vy", "vz"):
        a = getattr(s, k).copy()
        a[fast] = a[fast] * 50.0
        setattr(s, k, a)
    parts.append(s)
    # sizes around warp / block boundaries
    for n in (20, 21, 31, 32, 33, 63, 64, 65, 255, 256, 257, 1023, 1024, 1025):
        if n <= sizes[big]:
            parts.append(one(big, n))
    return concat(parts)


def main() -> None:
    import oracle as O
    O.build()
    cases = []
    L = synth.generate("cfg1")
    cases.append(("cfg1_slice", L.select(np.arange(0, L.nhalo, 2))))
    cases.append(("edge_cases", edge_cases(L)))
    M = synth.generate("cfg3", scale=0.0003, max_particles=3000, multimass=True)
    cases.append(("multimass_slice", M))
    S = synth.generate("cfg2", scale=0.1, max_particles=12000)
    hosts = [i for i in range(S.nhalo) if np.diff(S.off)[i] > 10000][:1]
    if hosts:
        h = hosts[0]
        cases.append(("subhalo_lists", S.select([h, S.nhalo - 3, S.nhalo - 2, S.nhalo - 1])))
    for name, lists in cases:
        p = synth.params_for({"multimass_slice": M, "subhalo_lists": S}.get(name, L))
        res = O.run_reference(p, lists)
        save_case(name, p, lists, res)
        print(name, lists.nhalo, lists.n, "kept", res.stats["n_kept"],
              os.path.getsize(os.path.join(HERE, name + ".npz")))


def gather_cases():
    """Inputs of the particle-gather fixtures: a cfg1 snapshot (its lists
    plus 60,000 uniform particles) and the hand-built edge cases."""
    L = synth.generate("cfg1")
    return [("gather_cfg1", synth.snapshot_from_lists(L, 60000)), ("gather_edges", synth.gather_edge_snapshot())]


def make_gather() -> None:
    """The reference's own SFC gather (ahf_halos_sfc_gatherParts) on each
    case; lists stored in the reference's order."""
    import oracle as O
    O.build()
    for name, S in gather_cases():
        off, idx = O.gather_reference(S.x, S.y, S.z, S.cx, S.cy, S.cz, S.rad)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), x=S.x, y=S.y, z=S.z, cx=S.cx, cy=S.cy, cz=S.cz,
                            rad=S.rad, off=off, idx=idx)
        print(name, S.n, S.nhalo, "gathered", int(off[-1]), os.path.getsize(os.path.join(HERE, name + ".npz")))


def make_writer() -> None:
    """The reference's own AHF_particles writer (ahf_io_WriteParticles) on the
    reference stage's kept lists of the cfg1 slice: inputs and the file's
    bytes (`data`), and the AHF_particles_bin bytes of the reference's
    -DAHFbinary build (ahf_binwrite_particles) on the same inputs
    (`data_bin`)."""
    import oracle as O
    O.build()
    L = synth.generate("cfg1")
    p = synth.params_for(L)
    res = O.run_reference(p, L)
    ids = (np.arange(L.n, dtype=np.uint64) * np.uint64(7919)) + np.uint64(10**12)
    order = np.argsort(-res.halo["npart"].astype(np.int64), kind="stable").astype(np.int64)
    data = O.write_particles_reference(ids, None, res.member_off, res.member, res.halo["npart"], order, 20)
    data_bin = O.write_particles_bin_reference(ids, res.member_off, res.member, res.halo["npart"], order, 20)
    np.savez_compressed(os.path.join(HERE, "writer_cfg1.npz"), ids=ids, member_off=res.member_off,
                        member=res.member, npart=res.halo["npart"], order=order, minpart=20,
                        data=np.frombuffer(data, np.uint8), data_bin=np.frombuffer(data_bin, np.uint8))
    print("writer_cfg1", len(data), os.path.getsize(os.path.join(HERE, "writer_cfg1.npz")))


def make_sfc() -> None:
    """The reference's own keying and particle sort (sfc_curve_calcKey at
    BITS_PER_DIMENSION, qsort by cmp_sfckey_part; main.c:342-356) on the cfg1
    snapshot of the gather fixture (its first 6000 particles) plus edge positions (0, 1 - 2^-24, 1.0)
    and repeated positions: inputs, sorted keys and the original index of
    each."""
    import oracle as O
    O.build()
    L = synth.generate("cfg1")
    S = synth.snapshot_from_lists(L, 20000, seed=9)
    x, y, z = (np.asarray(v, dtype=np.float32)[:6000].copy() for v in (S.x, S.y, S.z))
    x[:8], y[:8], z[:8] = 0.0, np.float32(1 - 2 ** -24), 1.0
    x[8:40], y[8:40], z[8:40] = x[100:132], y[100:132], z[100:132]
    keys, order = O.sfc_sort_reference(x, y, z)
    np.savez_compressed(os.path.join(HERE, "sfc_cfg1.npz"), x=x, y=y, z=z, keys=keys, order=order)
    print("sfc_cfg1", len(keys), os.path.getsize(os.path.join(HERE, "sfc_cfg1.npz")))


def make_radii() -> None:
    """The reference's own gather-radius loop (spatialRef2halos run on a
    two-level refinement tree, oracle/ref_radii.c) on 2500 haloes: counts
    with many ties, coincident and grid-aligned centres, R_vir above and
    below the radii; inputs, radii and the R_vir each halo carried."""
    import oracle as O
    O.build()
    rng = np.random.default_rng(21)
    n = 2500
    npart = np.floor(20 * rng.random(n) ** -1.3).astype(np.uint64)
    c = rng.random((3, n))
    c[:, :60] = np.round(c[:, :60], 2)
    c[:, 60:70] = c[:, 70:80]
    rvir = rng.random(n) * 0.004
    rvir[100:110] = 0.3
    maxg = 0.02
    rad, rv = O.gather_radii_reference(npart, c[0], c[1], c[2], rvir, maxg)
    np.savez_compressed(os.path.join(HERE, "radii_ref.npz"), npart=npart, cx=c[0], cy=c[1], cz=c[2], rvir=rv,
                        max_gather_rad_box=maxg, rad=rad)
    print("radii_ref", n, os.path.getsize(os.path.join(HERE, "radii_ref.npz")))


def amr_digest(zyx, dens) -> int:
    """First 8 bytes of the SHA-256 of a grid's nodes (int64 z, y, x) and
    densities (float64 of the float values)."""
    import hashlib
    h = hashlib.sha256(np.ascontiguousarray(zyx, np.int64).tobytes() + np.ascontiguousarray(dens, np.float64).tobytes())
    return int.from_bytes(h.digest()[:8], "little")


def make_amr() -> None:
    """The reference's own AMR hierarchy (oracle/ref_amr.c: gen_domgrids, ll,
    assign_npart, gen_AMRhierarchy) on the cfg1 snapshot of the gather
    fixture, for two domain grids: positions and (l1dim, nodes, particles)
    per grid; the 16^3 domain grid's TSC densities after assign_npart; and
    the nodes (z, y, x) of the first grid refined from the 32^3 domain grid."""
    import oracle as O
    O.build()
    L = synth.generate("cfg1")
    S = synth.snapshot_from_lists(L, 20000, seed=9)
    x, y, z = (np.asarray(v, dtype=np.float32) for v in (S.x, S.y, S.z))
    out = {"x": x, "y": y, "z": z}
    for tag, dom, mx in (("d16", 16, 4096), ("d32", 32, 256)):
        out[f"levels_{tag}"] = O.amr_levels_reference(x, y, z, dom, mx, 5.0, 5.0)
        out[f"params_{tag}"] = np.array([dom, mx, 5.0, 5.0])
    out["dens_d16"] = O.domain_dens_reference(x, y, z, 16)   # the 16^3 domain grid after assign_npart
    out["first_ref_d32"] = O.first_refinement_reference(x, y, z, 32, 5.0, 5.0).astype(np.int16)
    # every grid of the 16^3-domain hierarchy: a digest of its nodes (quad
    # order) and float densities
    out["level_digest_d16"] = np.array([amr_digest(*O.amr_nodes_reference(x, y, z, 16, 4096, 5.0, 5.0, lev))
                                        for lev in range(len(out["levels_d16"]))], dtype=np.uint64)
    np.savez_compressed(os.path.join(HERE, "amr_cfg1.npz"), **out)
    print("amr_cfg1", os.path.getsize(os.path.join(HERE, "amr_cfg1.npz")))


if __name__ == "__main__":
    main()
    make_gather()
    make_writer()
    make_sfc()
    make_radii()
    make_amr()
