"""Gather radii: the loop of spatialRef2halos (src/libahf/ahf_halos.c:2987-3051).

The loop sits at the end of spatialRef2halos, after the refinement tree has
been turned into haloes.  The restatement (oracle/ahf_oracle.c) is checked
against hand-worked cases, a second, vectorised numpy statement of the same
rule, and the reference itself: oracle/ref_radii.c runs the reference's
spatialRef2halos (compiled unchanged) on a two-level refinement tree that
yields the given haloes (live where the reference is compiled, and the
committed fixture tests/golden/radii_ref.npz).  GPU: the C ABI
(ahfgpu_gather_radii_device) equal to the oracle, bit for bit.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle
    oracle.build(ref=False)
    return oracle


def numpy_radii(npart, cx, cy, cz, rvir, maxg):
    """The rule written out independently: half the distance to the closest
    halo with strictly more particles, else max_rad; MAX with R_vir, MIN
    with max_rad = min(maxg, 1/4)."""
    maxr = min(maxg, 0.25)
    out = np.zeros(len(npart))
    for i in range(len(npart)):
        more = npart > npart[i]
        if not more.any():
            r = maxr
        else:
            d = []
            for a in (cx, cy, cz):
                t = np.abs(a[i] - a[more])
                d.append(np.where(t > 0.5, 1.0 - t, t))
            d2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
            r = np.sqrt(min(1e11, d2.min())) * 0.5
        r = max(r, rvir[i])
        out[i] = min(r, maxr)
    return out


def hand_case():
    npart = np.array([100, 50, 50, 10, 10, 7], np.uint64)
    cx = np.array([0.10, 0.30, 0.95, 0.02, 0.5, 0.31])
    cy = np.array([0.10, 0.10, 0.10, 0.10, 0.5, 0.10])
    cz = np.array([0.10, 0.10, 0.10, 0.10, 0.5, 0.10])
    rvir = np.array([0.001, 0.001, 0.2, 0.0, 0.0, 0.0])
    return npart, cx, cy, cz, rvir, 0.24


def test_gather_radii_hand_case():
    O = _oracle()
    npart, cx, cy, cz, rvir, maxg = hand_case()
    got = O.gather_radii_oracle(npart, cx, cy, cz, rvir, maxg)
    # 0: the largest -> max_rad; 1: nearest larger is 0, 0.2 away along x
    # -> 0.1; 2: its equal-count twin does not count, nearest larger is 0
    # across the periodic boundary (0.15) -> 0.075, raised to R_vir 0.2;
    # 3: nearest larger is 2, across the periodic boundary (0.07) -> 0.035;
    # 5: nearest larger is 1 (0.01) -> 0.005.  (Offsets along one axis:
    # sqrt(dx*dx) is |dx| exactly.)
    assert got[0] == 0.24
    assert got[1] == abs(0.30 - 0.10) * 0.5
    assert got[2] == 0.2
    assert got[3] == (1.0 - abs(0.02 - 0.95)) * 0.5
    assert got[5] == abs(0.31 - 0.30) * 0.5
    assert np.array_equal(got, numpy_radii(npart, cx, cy, cz, rvir, maxg))


def test_gather_radii_restatement_matches_numpy():
    O = _oracle()
    rng = np.random.default_rng(4)
    n = 1500
    npart = np.floor(20 * rng.random(n) ** -1.2).astype(np.uint64)   # many ties
    c = rng.random((3, n))
    rvir = rng.random(n) * 0.002
    got = O.gather_radii_oracle(npart, c[0], c[1], c[2], rvir, 0.3)
    assert np.array_equal(got, numpy_radii(npart, c[0], c[1], c[2], rvir, 0.3))


def test_gather_radii_restatement_matches_reference_live():
    O = _oracle()
    if not os.path.isfile(O.ref_radii_path()):
        pytest.skip("reference not compiled here")
    cases = [hand_case()]
    rng = np.random.default_rng(31)
    for n, maxg in ((1, 0.1), (2, 0.1), (4000, 0.3)):
        npart = np.floor(20 * rng.random(n) ** -1.2).astype(np.uint64)
        c = rng.random((3, n))
        c[:, : n // 10] = np.round(c[:, : n // 10], 1)          # coincident and grid-aligned centres
        cases.append((npart, c[0], c[1], c[2], rng.random(n) * 0.01, maxg))
    for npart, cx, cy, cz, rvir, maxg in cases:
        rad, rv = O.gather_radii_reference(npart, cx, cy, cz, rvir, maxg)
        assert rv[0] == -1.0 and np.array_equal(rv[1:], np.asarray(rvir, dtype=np.float64)[1:])
        assert np.array_equal(O.gather_radii_oracle(npart, cx, cy, cz, rv, maxg), rad)


def test_gather_radii_restatement_matches_reference_fixture():
    O = _oracle()
    d = np.load(os.path.join(HERE, "golden", "radii_ref.npz"))
    got = O.gather_radii_oracle(d["npart"], d["cx"], d["cy"], d["cz"], d["rvir"], float(d["max_gather_rad_box"]))
    assert np.array_equal(got, d["rad"])


@pytest.mark.gpu
def test_gpu_gather_radii_matches_oracle():
    import torch
    from ahf_gb300 import build, lib
    build.build()
    lib.init(0)
    O = _oracle()
    rng = np.random.default_rng(8)
    cases = [hand_case()]
    n = 20000
    npart = np.floor(20 * rng.random(n) ** -1.3).astype(np.uint64)
    c = rng.random((3, n))
    c[:, :50] = np.round(c[:, :50], 2)          # coincident and grid-aligned centres
    cases.append((npart, c[0], c[1], c[2], rng.random(n) * 0.003, 0.02))
    for npart, cx, cy, cz, rvir, maxg in cases:
        exp = O.gather_radii_oracle(npart, cx, cy, cz, rvir, maxg)
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a).astype(dt)).cuda()
        got = lib.gather_radii_device(t(npart, np.int64), t(cx, np.float64), t(cy, np.float64), t(cz, np.float64),
                                      t(rvir, np.float64), maxg).cpu().numpy()
        assert np.array_equal(got, exp)
