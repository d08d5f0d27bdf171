"""Seeded synthetic halo catalogues in the shapes of the five workloads.

AHF itself ships no data; these generators stand in for its snapshots.  Every
halo is an NFW sphere (concentration c = 10 * 10**N(0, 0.1 dex), truncated at
R_vir with R_vir from M = 200 rho_crit 4/3 pi R^3), radii drawn by inverting
m(x) = ln(1+x) - x/(1+x), isotropic Maxwellian velocities with
sigma = sqrt(G M / (2 R_vir)).  The first 10 % of each halo's NFW particles
have their velocities scaled by 3 (unbound interlopers).  Each halo's
particle list also holds uniform background particles (mean matter density,
sigma = 100 km/s) out to 1.5 R_vir, which is the role of AHF's gather radius.
Hosts above 1e4 particles (workloads "cfg2"/"cfg5") carry 3 NFW subhaloes at
0.3-0.8 R_vir with 1-5 % of the host mass; subhaloes are haloes of their own
whose lists also pick up the host particles inside their 1.5 R_vir.

Units are AHF's internal ones: positions in box units [0,1), velocities as
AHF momenta (km/s divided by v_fac = 100 * boxsize / a), masses as weights
(mass / lightest mass, only with ``multimass``).  The cosmology is
Omega_m = 0.3, Omega_L = 0.7, z = 0, Dvir = 200 (rho_crit), VescTune = 1.5,
NminPerHalo = 20, giving a particle mass of 3.97e10 Msun/h in every box.

Workloads (the names used by bench.py and the tests):
  cfg1  64^3 / 50 Mpc/h, 20 haloes, M log-uniform in 1e12-1e14 Msun/h
  cfg2  256^3 / 200 Mpc/h, 2,000 haloes, N_p ~ N^-1.9 on [20, 1e6], subhaloes
  cfg3  1e5 direct lists, N_p ~ N^-1.56 on [20, 2e6] (sum ~ 4e8), 500 Mpc/h box
  cfg4  512^3 / 400 Mpc/h, 40,000 cfg1-like haloes
  cfg5  1024^3 / 800 Mpc/h, 5e5 haloes, N^-1.9 on [20, 1e6], subhaloes
The generator runs on torch (CPU for tests, CUDA for the large workloads) and
returns numpy or torch arrays.

`box_snapshot` builds the whole periodic box of a snapshot workload (cfg1,
cfg2, cfg4, cfg5: ngrid^3 equal-mass particles, the haloes' NFW particles
and a uniform background for the rest) and `write_gadget1` writes it as a
GADGET-1 file (AHF ic_filetype 60) with an AHF.input beside it, for runs of
the whole AHF program.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

GRAV = 4.3006485e-9     # Mpc km^2 / (Msun s^2)
H0 = 100.0
RHOC0 = 3.0 * H0 * H0 / 8.0 / math.pi / GRAV   # Msun/h / (Mpc/h)^3
OMEGA_M = 0.3
OMEGA_L = 0.7


@dataclass
class HaloLists:
    """CSR particle lists, one per halo (the ahfgpu_batch contents)."""
    off: np.ndarray                 # uint64 [nhalo+1]
    x: object
    y: object
    z: object
    vx: object
    vy: object
    vz: object
    w: object                       # float32 weights or None
    gidx: object                    # uint64 (int64 in torch) entry ids
    cx: np.ndarray
    cy: np.ndarray
    cz: np.ndarray
    boxsize: float
    pmass: float
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def nhalo(self) -> int:
        return len(self.off) - 1

    @property
    def n(self) -> int:
        return int(self.off[-1])

    def to_numpy(self) -> "HaloLists":
        def cv(a, dt):
            if a is None:
                return None
            if isinstance(a, torch.Tensor):
                a = a.detach().cpu().numpy()
            return np.ascontiguousarray(a).astype(dt, copy=False)
        return HaloLists(self.off, cv(self.x, np.float32), cv(self.y, np.float32), cv(self.z, np.float32),
                         cv(self.vx, np.float32), cv(self.vy, np.float32), cv(self.vz, np.float32),
                         cv(self.w, np.float32), cv(self.gidx, np.uint64), self.cx, self.cy, self.cz,
                         self.boxsize, self.pmass, self.name, dict(self.meta))

    def select(self, halos) -> "HaloLists":
        """Sub-batch of the given halo indices (numpy or torch arrays; the
        sub-batch keeps the array kind and device)."""
        halos = np.asarray(halos, dtype=np.int64)
        counts = (self.off[halos + 1] - self.off[halos]).astype(np.int64)
        off = np.zeros(len(halos) + 1, np.uint64)
        off[1:] = np.cumsum(counts)
        idx = np.concatenate([np.arange(self.off[h], self.off[h + 1], dtype=np.int64) for h in halos]) \
            if len(halos) else np.zeros(0, np.int64)
        if isinstance(self.x, torch.Tensor):
            idx = torch.as_tensor(idx, device=self.x.device)
        g = lambda a: None if a is None else a[idx]
        return HaloLists(off, g(self.x), g(self.y), g(self.z), g(self.vx), g(self.vy), g(self.vz),
                         g(self.w), g(self.gidx), self.cx[halos].copy(), self.cy[halos].copy(),
                         self.cz[halos].copy(), self.boxsize, self.pmass, self.name, dict(self.meta))


def ahf_params(boxsize: float, pmass: float, a: float = 1.0, Dvir: float = 200.0,
               VescTune: float = 1.5, MINPART: int = 20, omega0: float = OMEGA_M,
               lambda0: float = OMEGA_L):
    """The ahfgpu_params values, computed as src/libahf/ahf_halos.c:199-221 does
    (t_unit = 1/H0 from src/startrun.c:547; calc_Hubble, calc_rho_crit and the
    UserDvir branch of calc_virial from src/libutility/cosmology.c)."""
    from .abi import Params
    t_unit = 1.0 / H0
    hub = H0 * math.sqrt(lambda0 * (1. - 1. / (a * a)) + omega0 * (1. / (a * a * a) - 1. / (a * a)) + 1. / (a * a))
    rho_crit = 3. * (hub * hub) / 8. / math.pi / GRAV
    p = Params()
    p.VescTune = VescTune
    p.MINPART = MINPART
    p.ovlim = Dvir
    p.rho_vir = (a * a * a) * rho_crit
    p.r_fac = boxsize * a
    p.x_fac = boxsize
    p.v_fac = boxsize / t_unit / a
    p.m_fac = pmass
    p.rho_fac = pmass / (boxsize * boxsize * boxsize)
    p.phi_fac = GRAV * pmass / (boxsize * a)
    p.Hubble = hub
    return p


CONFIGS = {
    "cfg1": dict(box=50.0, ngrid=64, nhalo=20, dist="logmass", mlo=1e12, mhi=1e14, subs=False, seed=12346),
    "cfg2": dict(box=200.0, ngrid=256, nhalo=2000, dist="power", alpha=1.9, nlo=20, nhi=1e6, subs=True,
                 seed=12347),
    "cfg3": dict(box=500.0, ngrid=None, nhalo=100000, dist="power", alpha=1.56, nlo=20, nhi=2e6, subs=False,
                 seed=12348),
    "cfg4": dict(box=400.0, ngrid=512, nhalo=40000, dist="logmass", mlo=1e12, mhi=1e14, subs=False, seed=12349),
    "cfg5": dict(box=800.0, ngrid=1024, nhalo=500000, dist="power", alpha=1.9, nlo=20, nhi=1e6, subs=True,
                 seed=12350),
}
PMASS = OMEGA_M * RHOC0 * 50.0 ** 3 / 64 ** 3      # 3.97e10 Msun/h in every box


def _power_counts(rng, n, alpha, lo, hi):
    u = rng.random(n)
    a1 = 1.0 - alpha
    return np.floor((lo ** a1 + u * (hi ** a1 - lo ** a1)) ** (1.0 / a1)).astype(np.int64)


def _nfw_m(x):
    return torch.log1p(x) - x / (1.0 + x)


def _nfw_inverse(u, c, iters=40):
    """x in [0,c] with m(x) = u m(c), by bisection in log x (float32)."""
    target = u * _nfw_m(c)
    lo = torch.full_like(u, -12.0)
    hi = torch.log(c)
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        f = _nfw_m(torch.exp(mid)) - target
        below = f < 0
        lo = torch.where(below, mid, lo)
        hi = torch.where(below, hi, mid)
    return torch.exp(0.5 * (lo + hi))


def _halo_table(cfg, nhalo, rng, pmass):
    """Per-halo (N_p, R_vir, c, sigma, centre, bulk velocity) in Mpc/h, km/s."""
    if cfg["dist"] == "logmass":
        m = 10 ** rng.uniform(math.log10(cfg["mlo"]), math.log10(cfg["mhi"]), nhalo)
        npart = np.maximum(np.round(m / pmass).astype(np.int64), 1)
    else:
        npart = _power_counts(rng, nhalo, cfg["alpha"], cfg["nlo"], cfg["nhi"])
    mass = npart * pmass
    rvir = (3.0 * mass / (4.0 * math.pi * 200.0 * RHOC0)) ** (1.0 / 3.0)
    conc = 10.0 * 10 ** rng.normal(0.0, 0.1, nhalo)
    sigma = np.sqrt(GRAV * mass / (2.0 * rvir))
    centre = rng.random((nhalo, 3)) * cfg["box"]
    bulk = rng.normal(0.0, 200.0, (nhalo, 3))
    return dict(npart=npart, mass=mass, rvir=rvir, conc=conc, sigma=sigma, centre=centre, bulk=bulk,
                host=-np.ones(nhalo, np.int64))


def _add_subhalos(tab, rng):
    """3 subhaloes per host above 1e4 particles (1-5 % of the host mass at
    0.3-0.8 R_vir, bulk velocity from the host Maxwellian)."""
    hosts = np.nonzero(tab["npart"] > 10000)[0]
    rows = {k: [v] for k, v in tab.items()}
    for h in hosts:
        for _ in range(3):
            frac = rng.uniform(0.01, 0.05)
            n = max(int(tab["npart"][h] * frac), 20)
            m = n * (tab["mass"][h] / tab["npart"][h])
            rv = (3.0 * m / (4.0 * math.pi * 200.0 * RHOC0)) ** (1.0 / 3.0)
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            pos = tab["centre"][h] + d * rng.uniform(0.3, 0.8) * tab["rvir"][h]
            rows["npart"].append(np.array([n]))
            rows["mass"].append(np.array([m]))
            rows["rvir"].append(np.array([rv]))
            rows["conc"].append(np.array([10.0 * 10 ** rng.normal(0.0, 0.1)]))
            rows["sigma"].append(np.array([math.sqrt(GRAV * m / (2.0 * rv))]))
            rows["centre"].append(pos[None, :])
            rows["bulk"].append((tab["bulk"][h] + rng.normal(0.0, tab["sigma"][h], 3))[None, :])
            rows["host"].append(np.array([h]))
    return {k: np.concatenate(v) for k, v in rows.items()}


def _sample_spheres(tab, sel, nfw_counts, bg_counts, gen, device):
    """Particles (positions in Mpc/h relative to the box, velocities km/s) of
    the NFW + background spheres of haloes `sel`; returns per-particle
    tensors ordered halo by halo and the per-halo counts."""
    counts = nfw_counts + bg_counts
    N = int(counts.sum())
    cnt_t = torch.as_tensor(counts, device=device)
    hid = torch.repeat_interleave(torch.arange(len(sel), device=device), cnt_t)
    start = torch.as_tensor(np.concatenate([[0], np.cumsum(counts)[:-1]]), device=device)
    local = torch.arange(N, device=device) - start[hid]
    nfw_t = torch.as_tensor(nfw_counts, device=device)
    is_nfw = local < nfw_t[hid]
    is_int = local < torch.as_tensor(np.ceil(0.1 * nfw_counts).astype(np.int64), device=device)[hid]
    f32 = dict(device=device, dtype=torch.float32)
    rvir = torch.as_tensor(tab["rvir"][sel], **f32)[hid]
    conc = torch.as_tensor(tab["conc"][sel], **f32)[hid]
    sig = torch.as_tensor(tab["sigma"][sel], **f32)[hid]
    u = torch.rand(N, generator=gen, **f32).clamp_(1e-7, 1.0)
    x = _nfw_inverse(u, conc)
    r_nfw = x * (rvir / conc)
    r_bg = 1.5 * rvir * torch.rand(N, generator=gen, **f32).pow(1.0 / 3.0)
    r = torch.where(is_nfw, r_nfw, r_bg)
    ct = 2.0 * torch.rand(N, generator=gen, **f32) - 1.0
    ph = 2.0 * math.pi * torch.rand(N, generator=gen, **f32)
    st = torch.sqrt((1.0 - ct * ct).clamp_min(0.0))
    d = torch.stack([st * torch.cos(ph), st * torch.sin(ph), ct], 1)
    cen = torch.as_tensor(tab["centre"][sel], device=device, dtype=torch.float64)[hid]
    pos = cen + (r[:, None] * d).to(torch.float64)
    v = torch.randn(N, 3, generator=gen, **f32)
    scale = torch.where(is_nfw, sig * torch.where(is_int, 3.0, 1.0), torch.full_like(sig, 100.0))
    bulk = torch.as_tensor(tab["bulk"][sel], **f32)[hid]
    vel = v * scale[:, None] + torch.where(is_nfw[:, None], bulk, torch.zeros_like(bulk))
    return pos, vel, counts


def _to_ahf_units(pos, vel, box, v_fac):
    """Mpc/h, km/s -> box units in [0,1) (float32) and AHF momenta (float32)."""
    pb = torch.remainder(pos / box, 1.0)
    pb = torch.where(pb >= 1.0, torch.zeros_like(pb), pb)
    pf = pb.to(torch.float32)
    pf = torch.where(pf >= 1.0, torch.zeros_like(pf), pf)
    mom = (vel.to(torch.float64) / v_fac).to(torch.float32)
    return pf, mom


def generate(name: str, scale: float = 1.0, device: str = "cpu", multimass: bool = False,
             seed: int | None = None, max_particles: int | None = None, as_numpy: bool = True) -> HaloLists:
    """Build the particle lists of workload `name` (see module docstring).

    scale multiplies the number of haloes (small test cases); max_particles
    caps the per-halo count (keeps test cases small)."""
    cfg = dict(CONFIGS[name])
    rng = np.random.default_rng(cfg["seed"] if seed is None else seed)
    nhalo = max(1, int(round(cfg["nhalo"] * scale)))
    box = cfg["box"]
    pmass = PMASS
    tab = _halo_table(cfg, nhalo, rng, pmass)
    if max_particles is not None:
        tab["npart"] = np.minimum(tab["npart"], max_particles)
    if cfg["subs"]:
        tab = _add_subhalos(tab, rng)
    nh = len(tab["npart"])
    bg_density = OMEGA_M * RHOC0 / pmass
    nbg = rng.poisson(bg_density * 4.0 / 3.0 * math.pi * (1.5 * tab["rvir"]) ** 3)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(rng.integers(1 << 62)))
    v_fac = box * H0          # a = 1
    if cfg["subs"] and np.any(tab["host"] >= 0):
        sel = np.arange(nh)
        pos, vel, counts = _sample_spheres(tab, sel, tab["npart"], nbg, gen, device)
        # subhalo particles join their host's list; host particles inside a
        # subhalo's 1.5 R_vir join the subhalo's list.
        starts = np.concatenate([[0], np.cumsum(counts)])
        parts_pos = [pos[starts[h]:starts[h + 1]] for h in range(nh)]
        parts_vel = [vel[starts[h]:starts[h + 1]] for h in range(nh)]
        own_pos, own_vel = list(parts_pos), list(parts_vel)
        for s in np.nonzero(tab["host"] >= 0)[0]:
            h = tab["host"][s]
            parts_pos[h] = torch.cat([parts_pos[h], own_pos[s]])
            parts_vel[h] = torch.cat([parts_vel[h], own_vel[s]])
            cen = torch.as_tensor(tab["centre"][s], device=device, dtype=torch.float64)
            near = ((own_pos[h] - cen) ** 2).sum(1) < (1.5 * tab["rvir"][s]) ** 2
            parts_pos[s] = torch.cat([parts_pos[s], own_pos[h][near]])
            parts_vel[s] = torch.cat([parts_vel[s], own_vel[h][near]])
        counts = np.array([len(p) for p in parts_pos], np.int64)
        chunks = [(torch.cat(parts_pos), torch.cat(parts_vel))]
    else:
        # chunks of haloes (bounded temporary memory for the 4e8-particle case)
        counts = (tab["npart"] + nbg).astype(np.int64)
        chunks = []
        h0 = 0
        budget = 40_000_000
        while h0 < nh:
            h1 = h0 + 1
            acc = counts[h0]
            while h1 < nh and acc + counts[h1] <= budget:
                acc += counts[h1]
                h1 += 1
            sel = np.arange(h0, h1)
            pos, vel, _ = _sample_spheres(tab, sel, tab["npart"][sel], nbg[sel], gen, device)
            chunks.append(_to_ahf_units(pos, vel, box, v_fac))
            del pos, vel
            h0 = h1
    off = np.zeros(nh + 1, np.uint64)
    off[1:] = np.cumsum(counts)
    if cfg["subs"] and np.any(tab["host"] >= 0):
        pf, mom = _to_ahf_units(chunks[0][0], chunks[0][1], box, v_fac)
    else:
        pf = torch.cat([c[0] for c in chunks]) if len(chunks) > 1 else chunks[0][0]
        mom = torch.cat([c[1] for c in chunks]) if len(chunks) > 1 else chunks[0][1]
    del chunks
    N = int(off[-1])
    w = None
    if multimass:
        heavy = torch.rand(N, generator=gen, device=device) < 0.15
        w = torch.where(heavy, 5.0, 1.0).to(torch.float32)
    gidx = torch.arange(N, device=device, dtype=torch.int64)
    cen = tab["centre"] / box
    cen = np.mod(cen, 1.0)
    out = HaloLists(off, pf[:, 0].contiguous(), pf[:, 1].contiguous(), pf[:, 2].contiguous(),
                    mom[:, 0].contiguous(), mom[:, 1].contiguous(), mom[:, 2].contiguous(), w, gidx,
                    np.ascontiguousarray(cen[:, 0]), np.ascontiguousarray(cen[:, 1]),
                    np.ascontiguousarray(cen[:, 2]), box, pmass, name,
                    dict(scale=scale, multimass=multimass, nhalo_primary=nhalo))
    return out.to_numpy() if as_numpy else out


def parity_halos(n_in: np.ndarray, largest: int = 20, sample_particles: float = 2e7, seed: int = 31) -> np.ndarray:
    """Haloes for a full-size parity check, ascending: the `largest` longest
    lists plus a seeded random choice of the others holding about
    `sample_particles` entries (drawn uniformly over haloes, so the sample
    follows the batch's size mix)."""
    n_in = np.asarray(n_in, np.int64)
    top = np.argsort(-n_in, kind="stable")[:largest]
    rest = np.setdiff1d(np.arange(len(n_in)), top)
    rng = np.random.default_rng(seed)
    perm = rest[rng.permutation(len(rest))]
    k = int(np.searchsorted(np.cumsum(n_in[perm]), sample_particles)) + 1 if len(perm) else 0
    return np.sort(np.concatenate([top, perm[:k]]))


def params_for(lists: HaloLists, **kw):
    return ahf_params(lists.boxsize, lists.pmass, **kw)


@dataclass
class Snapshot:
    """Particles of a periodic box plus halo centres and gather radii (the
    inputs of AHF's particle gather)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    w: object
    cx: np.ndarray
    cy: np.ndarray
    cz: np.ndarray
    rad: np.ndarray

    @property
    def n(self) -> int:
        return len(self.x)

    @property
    def nhalo(self) -> int:
        return len(self.cx)


def snapshot_from_lists(lists: HaloLists, n_background: int, seed: int = 7, shuffle: bool = True) -> Snapshot:
    """A snapshot made of every particle of the lists (each list is its own
    NFW sphere plus background out to 1.5 R_vir) and `n_background` uniform
    particles (sigma 100 km/s) over the whole box, in a seeded random order
    (shuffle=False: the lists' particles in list order, then the uniform ones).
    Each halo's gather radius is the largest periodic distance of its own
    list's particles from its centre (<= 1.5 R_vir)."""
    L = lists.to_numpy() if not isinstance(lists.x, np.ndarray) else lists
    rng = np.random.default_rng(seed)
    vsig = 100.0 / (L.boxsize * H0)
    bx = rng.random((n_background, 3)).astype(np.float32)
    bv = (rng.standard_normal((n_background, 3)) * vsig).astype(np.float32)
    pos = np.concatenate([np.stack([L.x, L.y, L.z], 1).astype(np.float32), bx])
    vel = np.concatenate([np.stack([L.vx, L.vy, L.vz], 1).astype(np.float32), bv])
    w = None
    if L.w is not None:
        w = np.concatenate([np.asarray(L.w, np.float32), np.ones(n_background, np.float32)])
    perm = rng.permutation(len(pos)) if shuffle else np.arange(len(pos))
    pos, vel = pos[perm], vel[perm]
    if w is not None:
        w = w[perm]
    off = L.off.astype(np.int64)
    rad = np.zeros(L.nhalo)
    for h in range(L.nhalo):
        s = slice(off[h], off[h + 1])
        if off[h + 1] == off[h]:
            continue
        d2 = np.zeros(off[h + 1] - off[h])
        for a, c in ((L.x, L.cx), (L.y, L.cy), (L.z, L.cz)):
            d = np.abs(a[s].astype(np.float64) - c[h])
            d = np.where(d > 0.5, 1.0 - d, d)
            d2 += d * d
        rad[h] = float(np.sqrt(d2.max()))
    return Snapshot(np.ascontiguousarray(pos[:, 0]), np.ascontiguousarray(pos[:, 1]), np.ascontiguousarray(pos[:, 2]),
                    np.ascontiguousarray(vel[:, 0]), np.ascontiguousarray(vel[:, 1]), np.ascontiguousarray(vel[:, 2]),
                    w, np.asarray(L.cx, np.float64).copy(), np.asarray(L.cy, np.float64).copy(),
                    np.asarray(L.cz, np.float64).copy(), rad)


def gather_edge_snapshot(seed: int = 11) -> Snapshot:
    """Hand-built gather cases: centres on box faces, edges and corners
    (periodic wrap), a zero radius, a radius above 0.5 (the whole box along
    every axis), two haloes with the same centre, a centre exactly on a
    particle, particles exactly on the box's lower faces."""
    rng = np.random.default_rng(seed)
    n = 40000
    pos = rng.random((n, 3)).astype(np.float32)
    pos[:50, 0] = 0.0
    pos[50:100, 1] = 0.0
    pos[100:120] = 0.0
    vel = (rng.standard_normal((n, 3)) * 0.01).astype(np.float32)
    cen = np.array([[0.0, 0.5, 0.5], [0.999, 0.999, 0.999], [0.0, 0.0, 0.0], [0.5, 0.0, 0.999],
                    [0.3, 0.3, 0.3], [0.3, 0.3, 0.3], [0.25, 0.75, 0.5], [0.6, 0.2, 0.9],
                    [float(pos[500, 0]), float(pos[500, 1]), float(pos[500, 2])], [0.01, 0.99, 0.5]])
    rad = np.array([0.05, 0.08, 0.03, 0.1, 0.0, 0.04, 0.6, 0.02, 0.015, 0.12])
    return Snapshot(np.ascontiguousarray(pos[:, 0]), np.ascontiguousarray(pos[:, 1]), np.ascontiguousarray(pos[:, 2]),
                    np.ascontiguousarray(vel[:, 0]), np.ascontiguousarray(vel[:, 1]), np.ascontiguousarray(vel[:, 2]),
                    None, np.ascontiguousarray(cen[:, 0]), np.ascontiguousarray(cen[:, 1]),
                    np.ascontiguousarray(cen[:, 2]), rad)


@dataclass
class BoxSnapshot:
    """A whole periodic box: positions in Mpc/h in [0, box), peculiar
    velocities in km/s, 32-bit ids, equal particle masses (Msun/h)."""
    pos: np.ndarray
    vel: np.ndarray
    ids: np.ndarray
    box: float
    pmass: float
    nhalo: int


def box_snapshot(name: str, scale: float = 1.0, seed: int | None = None) -> BoxSnapshot:
    """ngrid^3 particles: the NFW particles of the workload's haloes (and
    subhaloes), truncated at R_vir, 10 % interlopers with v x 3, then a
    uniform background (sigma = 100 km/s per axis) for the rest of the box;
    ids are a seeded permutation of 1..N, the file order a seeded shuffle.
    `scale` multiplies the number of haloes."""
    cfg = dict(CONFIGS[name])
    rng = np.random.default_rng(cfg["seed"] if seed is None else seed)
    nhalo = max(1, int(round(cfg["nhalo"] * scale)))
    box = cfg["box"]
    tab = _halo_table(cfg, nhalo, rng, PMASS)
    if cfg["subs"]:
        tab = _add_subhalos(tab, rng)
    nh = len(tab["npart"])
    gen = torch.Generator(device="cpu")
    gen.manual_seed(int(rng.integers(1 << 62)))
    pos, vel, counts = _sample_spheres(tab, np.arange(nh), tab["npart"], np.zeros(nh, np.int64), gen, "cpu")
    ntot = int(cfg["ngrid"]) ** 3
    nbg = ntot - int(counts.sum())
    if nbg < 0:
        raise ValueError(f"{name}: the haloes hold more than ngrid^3 particles")
    bpos = rng.random((nbg, 3)) * box
    bvel = rng.standard_normal((nbg, 3)) * 100.0
    P = np.concatenate([np.mod(pos.numpy(), box), bpos]).astype(np.float32)
    P[P >= box] = 0.0
    V = np.concatenate([vel.numpy().astype(np.float64), bvel]).astype(np.float32)
    perm = rng.permutation(ntot)
    ids = (rng.permutation(ntot) + 1).astype(np.uint32)
    return BoxSnapshot(np.ascontiguousarray(P[perm]), np.ascontiguousarray(V[perm]), ids, box, PMASS, nh)


def write_gadget1(path: str, snap: BoxSnapshot, outfile_prefix: str, input_path: str,
                  omega0: float = OMEGA_M, lambda0: float = OMEGA_L, write_snapshot: bool = True) -> None:
    """The snapshot as a single GADGET-1 file (Fortran-record blocks: the
    256-byte header, POS, VEL, ID; one particle type, its mass in the header;
    lengths in Mpc/h, masses in 1e10 Msun/h, a = 1; skipped when not
    `write_snapshot`) and an AHF.input for it
    (ic_filetype 60, LgridDomain 64, NperDomCell = NperRefCell = 5,
    VescTune 1.5, NminPerHalo 20, RhoVir 0, Dvir 200, MaxGatherRad 3)."""
    import struct
    n = len(snap.ids)
    hdr = struct.pack("<6i", 0, n, 0, 0, 0, 0)
    hdr += struct.pack("<6d", 0.0, snap.pmass / 1e10, 0.0, 0.0, 0.0, 0.0)
    hdr += struct.pack("<dd", 1.0, 0.0)              # expansion, redshift
    hdr += struct.pack("<ii", 0, 0)                  # flag_sfr, flag_feedback
    hdr += struct.pack("<6I", 0, n, 0, 0, 0, 0)      # npartTotal
    hdr += struct.pack("<ii", 0, 1)                  # flag_cooling, num_files
    hdr += struct.pack("<4d", snap.box, omega0, lambda0, 0.7)
    hdr += b"\0" * (256 - len(hdr))

    def block(f, data: bytes):
        f.write(struct.pack("<i", len(data)))
        f.write(data)
        f.write(struct.pack("<i", len(data)))
    if write_snapshot:
        with open(path, "wb") as f:
            block(f, hdr)
            block(f, np.ascontiguousarray(snap.pos, "<f4").tobytes())
            block(f, np.ascontiguousarray(snap.vel, "<f4").tobytes())
            block(f, np.ascontiguousarray(snap.ids, "<u4").tobytes())
    with open(input_path, "w") as f:
        f.write("[AHF]\n"
                f"ic_filename       = {path}\n"
                "ic_filetype       = 60\n"
                f"outfile_prefix    = {outfile_prefix}\n"
                "LgridDomain       = 64\n"
                "LgridMax          = 16777216\n"
                "NperDomCell       = 5.0\n"
                "NperRefCell       = 5.0\n"
                "VescTune          = 1.5\n"
                "NminPerHalo       = 20\n"
                "RhoVir            = 0\n"
                "Dvir              = 200\n"
                "MaxGatherRad      = 3.0\n"
                "LevelDomainDecomp = 6\n"
                "NcpuReading       = 1\n"
                "\n[GADGET]\n"
                "GADGET_LUNIT      = 1.0\n"
                "GADGET_MUNIT      = 1e10\n")
