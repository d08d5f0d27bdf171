"""Result comparison used by every parity test.

Policy (the bar each test states):
  * kept particle lists (member_off, member): identical, in order;
  * npart, nbins and the stage flags: identical;
  * scalar properties: relative tolerance `rtol` (1e-10 for the FP64 forms,
    1e-6 for the FP32-compensated form), absolute floor `atol`; the halo's
    AngMom components and a profile bin's angular momentum components
    relative to that vector's norm (a
    component near zero is the difference of large terms, and carries the
    rounding of the whole vector in the reference's own sums too);
  * eigenvectors (E1..E3, per bin too): compared up to sign through
    |e_a . e_b| >= 1 - etol, skipped where two eigenvalues are within 1e-6
    relative of each other (the eigenvector is then not defined);
  * cNFW / cR1 are bisection results on a 1e-3 grid: absolute 2e-3.
"""
from __future__ import annotations

import numpy as np

from ahf_gb300.abi import HALO_STAGE_MASK, PROF_FIELDS

SCALARS = ["M_vir", "R_vir", "ovdens", "Phi0", "vel", "sigV", "v_esc2", "V2_max", "R_max", "r2",
           "lambda_", "lambdaE", "Ekin", "Epot", "SurfP", "pos_com", "com_offset", "pos_mbp", "vel_mbp",
           "mbp_offset", "AngMom", "axis", "fMhires", "R1"]
NORTH_STAR = ["M_vir", "R_vir", "V2_max", "R_max", "pos_com", "vel", "sigV", "lambda_", "lambdaE"]
EIG = ["E1", "E2", "E3"]


def rel_err(a, b, atol=0.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    scale = np.maximum(np.abs(b), atol if atol > 0 else 1e-300)
    both_nan = np.isnan(a) & np.isnan(b)
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    e = np.where(both_nan | both_inf | (d == 0), 0.0, d / scale)
    return e


def _halo(res, k):
    return res.halo[k] if hasattr(res, "halo") else res["halo_" + k]


def _get(res, k):
    return getattr(res, k) if hasattr(res, k) else res[k]


def compare(got, exp, rtol=1e-10, atol=1e-300, etol=1e-8, check_eig=True, skip_order=False):
    """Return a list of failure strings (empty = pass)."""
    bad = []
    mo_g, mo_e = _get(got, "member_off"), _get(exp, "member_off")
    if not np.array_equal(mo_g, mo_e):
        nd = int(np.sum(np.diff(mo_g.astype(np.int64)) != np.diff(mo_e.astype(np.int64))))
        bad.append(f"member counts differ in {nd} haloes")
    else:
        m_g, m_e = _get(got, "member"), _get(exp, "member")
        if skip_order:
            for h in range(len(mo_g) - 1):
                a = np.sort(m_g[mo_g[h]:mo_g[h + 1]])
                b = np.sort(m_e[mo_e[h]:mo_e[h + 1]])
                if not np.array_equal(a, b):
                    bad.append(f"member set differs in halo {h}")
                    break
        elif not np.array_equal(m_g, m_e):
            bad.append(f"member order/ids differ at {int(np.argmax(m_g != m_e))}")
    for k in ("npart", "nbins"):
        if not np.array_equal(_halo(got, k), _halo(exp, k)):
            bad.append(f"{k} differs in {int(np.sum(_halo(got, k) != _halo(exp, k)))} haloes")
    fg = _halo(got, "flags") & HALO_STAGE_MASK
    fe = _halo(exp, "flags") & HALO_STAGE_MASK
    if not np.array_equal(fg, fe):
        bad.append(f"stage flags differ in {int(np.sum(fg != fe))} haloes")
    ran = (_halo(exp, "flags") & 0x020) != 0
    nob = (_halo(exp, "flags") & 0x200) != 0
    for k in SCALARS:
        a, b = _halo(got, k), _halo(exp, k)
        e = rel_err(a, b, atol)
        if k == "R_vir":
            e = e[~nob] if e.ndim == 1 else e[~nob]
        if k == "AngMom":
            # components against the vector's norm (see the profile L below)
            nrm = np.linalg.norm(np.asarray(b, np.float64).reshape(-1, 3), axis=1, keepdims=True)
            d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).reshape(-1, 3)
            e = np.where(d == 0, 0.0, d / np.maximum(nrm, 1e-300))
        if e.size and np.max(e) > rtol:
            i = int(np.argmax(e.reshape(len(e), -1).max(1)))
            bad.append(f"{k}: max rel err {np.max(e):.3e} (halo {i})")
    for k in ("cNFW", "cR1"):
        d = np.abs(_halo(got, k) - _halo(exp, k))
        if d.size and np.max(d) > 2e-3:
            bad.append(f"{k}: max abs err {np.max(d):.3e}")
    if check_eig:
        axis = _halo(exp, "axis")
        for j, k in enumerate(EIG):
            a, b = _halo(got, k), _halo(exp, k)
            ok = _eig_ok(a, b, axis, j, etol) | ~ran
            if not np.all(ok):
                bad.append(f"{k}: {int(np.sum(~ok))} eigenvectors differ beyond sign")
    pg, pe = _get(got, "prof"), _get(exp, "prof")
    if pg.shape != pe.shape:
        bad.append(f"profile shape {pg.shape} vs {pe.shape}")
    elif pg.size:
        cols = [i for i, f in enumerate(PROF_FIELDS)
                if (not f.startswith("E") or f in ("Ekin", "Epot")) and f not in ("Lx", "Ly", "Lz")]
        e = rel_err(pg[:, cols], pe[:, cols], atol)
        if np.max(e) > rtol:
            c = cols[int(np.argmax(e.max(0)))]
            bad.append(f"profile {PROF_FIELDS[c]}: max rel err {np.max(e):.3e}")
        # a bin's angular momentum components against the bin's |L|: a
        # component that cancels to near zero carries the rounding of the
        # whole vector, in the reference's own sequential sums as in ours
        li = [PROF_FIELDS.index(f) for f in ("Lx", "Ly", "Lz")]
        norm = np.linalg.norm(pe[:, li], axis=1, keepdims=True)
        d = np.abs(pg[:, li] - pe[:, li])
        eL = np.where(d == 0, 0.0, d / np.maximum(norm, 1e-300))
        if np.max(eL) > rtol:
            bad.append(f"profile L: max err / |L_bin| {np.max(eL):.3e}")
        if check_eig:
            ax = pe[:, [PROF_FIELDS.index("axis1"), PROF_FIELDS.index("axis2"), PROF_FIELDS.index("axis3")]]
            for j, nm in enumerate(("E1", "E2", "E3")):
                ci = [PROF_FIELDS.index(nm + c) for c in "xyz"]
                ok = _eig_ok(pg[:, ci], pe[:, ci], ax, j, etol)
                if not np.all(ok):
                    bad.append(f"profile {nm}: {int(np.sum(~ok))} bins differ beyond sign")
    return bad


def _eig_ok(a, b, axis, j, etol):
    a = np.asarray(a, np.float64).reshape(-1, 3)
    b = np.asarray(b, np.float64).reshape(-1, 3)
    ax = np.asarray(axis, np.float64).reshape(-1, 3)
    dot = np.abs(np.sum(a * b, 1))
    zero = (np.abs(a).sum(1) == 0) & (np.abs(b).sum(1) == 0)
    # axis values are ratios sqrt(lambda_k/lambda_1); near-equal neighbours
    # leave the eigenvector undefined
    r = ax ** 2
    gaps = []
    if j > 0:
        gaps.append(np.abs(r[:, j] - r[:, j - 1]))
    if j < 2:
        gaps.append(np.abs(r[:, j] - r[:, j + 1]))
    degenerate = np.min(np.stack(gaps), 0) < 1e-6
    return zero | degenerate | (dot >= 1.0 - etol)


def compare_fp32c(got, exp, rtol_ns=1e-6, rtol_other=1e-4):
    """FP32-compensated bar: kept lists identical (in order), stage flags and
    counts identical, the spec properties (M_vir, R_vir, V2_max, R_max,
    pos_com, bulk velocity, sigV, lambda, lambdaE) within 1e-6 relative, the
    other per-halo properties and the profile rows within 1e-4 (relative, or
    absolute against the field's scale where the value itself is a small
    difference such as com_offset or an eigenvector component)."""
    bad = []
    mo_g, mo_e = _get(got, "member_off"), _get(exp, "member_off")
    if not np.array_equal(mo_g, mo_e):
        nd = int(np.sum(np.diff(mo_g.astype(np.int64)) != np.diff(mo_e.astype(np.int64))))
        bad.append(f"member counts differ in {nd} haloes")
    elif not np.array_equal(_get(got, "member"), _get(exp, "member")):
        bad.append("member ids/order differ")
    for k in ("npart", "nbins"):
        if not np.array_equal(_halo(got, k), _halo(exp, k)):
            bad.append(f"{k} differs in {int(np.sum(_halo(got, k) != _halo(exp, k)))} haloes")
    fg = _halo(got, "flags") & HALO_STAGE_MASK
    fe = _halo(exp, "flags") & HALO_STAGE_MASK
    if not np.array_equal(fg, fe):
        bad.append(f"stage flags differ in {int(np.sum(fg != fe))} haloes")
    nob = (_halo(exp, "flags") & 0x200) != 0
    for k in NORTH_STAR:
        e = rel_err(_halo(got, k), _halo(exp, k))
        if k == "R_vir":
            e = e[~nob]
        if e.size and np.max(e) > rtol_ns:
            ee = e.reshape(len(e), -1).max(1)
            i = int(np.argmax(ee))
            bad.append(f"{k}: max rel err {np.max(e):.3e} (north-star bar {rtol_ns:g}) halo {i}: "
                       f"{_halo(got, k)[i]} vs {_halo(exp, k)[i]}")
    loose = ["ovdens", "Phi0", "v_esc2", "r2", "Ekin", "Epot", "pos_mbp", "vel_mbp", "fMhires", "axis"]
    for k in loose:
        e = rel_err(_halo(got, k), _halo(exp, k), 1e-30)
        if e.size and np.max(e) > rtol_other:
            bad.append(f"{k}: max rel err {np.max(e):.3e}")
    for k, scale in (("com_offset", "R_vir"), ("mbp_offset", "R_vir")):
        d = np.abs(_halo(got, k) - _halo(exp, k)) / np.maximum(np.abs(_halo(exp, scale)), 1e-300)
        if d.size and np.max(d) > rtol_other:
            bad.append(f"{k}: max err/R_vir {np.max(d):.3e}")
    pg, pe = _get(got, "prof"), _get(exp, "prof")
    if pg.shape != pe.shape:
        bad.append(f"profile shape {pg.shape} vs {pe.shape}")
    elif pg.size:
        cols = [i for i, f in enumerate(PROF_FIELDS)
                if (not f.startswith("E") or f in ("Ekin", "Epot")) and f not in ("Lx", "Ly", "Lz")]
        e = rel_err(pg[:, cols], pe[:, cols], 1e-30)
        if np.max(e) > rtol_other:
            c = cols[int(np.argmax(e.max(0)))]
            bad.append(f"profile {PROF_FIELDS[c]}: max rel err {np.max(e):.3e}")
        # angular momentum per bin: absolute, against the halo's total |L|
        po = _get(exp, "prof_off")
        li = [PROF_FIELDS.index(f) for f in ("Lx", "Ly", "Lz")]
        worst = 0.0
        for h in range(len(po) - 1):
            a, b = int(po[h]), int(po[h + 1])
            if b <= a:
                continue
            scale = np.linalg.norm(pe[b - 1, li]) + 1e-300
            worst = max(worst, float(np.max(np.abs(pg[a:b, li] - pe[a:b, li])) / scale))
        if worst > rtol_other:
            bad.append(f"profile L: max abs err / |L_total| {worst:.3e}")
    return bad
