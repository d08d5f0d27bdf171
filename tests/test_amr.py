"""The AMR hierarchy (src/main.c:614-648, libamr_serial): oracle groundwork.

oracle/ref_amr.c runs the reference's own gen_domgrids, ll, assign_npart
and gen_AMRhierarchy (compiled unchanged) on float positions and reports
each grid's nodes per dimension, node count and particle count, and the
domain grid's TSC densities.  The committed fixture tests/golden/amr_cfg1.npz
holds its output on the cfg1 snapshot; the live reference must reproduce it
where it is compiled.  The hierarchy is restated in oracle/oracle_amr.c
(runs, segment-local neighbours, the refinement state machines, relink and
assign_npart in the reference's list order) and equal to the reference on
every grid: nodes in the reference's order and float densities bit for bit.
The domain grid's TSC density and the first refinement are also restated on
their own in oracle/ahf_oracle.c (a direct density sum and a stencil rule).  No GPU path of this row exists yet: these are the
numbers it will have to meet.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "amr_cfg1.npz")


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle
    oracle.build()
    return oracle


def test_fixture_levels_are_a_hierarchy():
    d = np.load(FIXTURE)
    n = len(d["x"])
    for tag in ("d16", "d32"):
        lv = d[f"levels_{tag}"]
        dom, mx = int(d[f"params_{tag}"][0]), int(d[f"params_{tag}"][1])
        assert lv[0, 0] == dom and lv[0, 1] == dom ** 3 and lv[0, 2] == n   # full domain grid, every particle
        assert np.all(lv[1:, 0] == 2 * lv[:-1, 0]) and lv[-1, 0] <= mx
        assert np.all(lv[1:, 2] <= n)


def test_refined_levels_do_not_depend_on_the_domain_grid():
    d = np.load(FIXTURE)
    a, b = d["levels_d16"], d["levels_d32"]
    common = np.intersect1d(a[1:, 0], b[1:, 0])
    common = common[common <= 256]
    assert len(common) >= 2
    for l1 in common:
        assert np.array_equal(a[a[:, 0] == l1], b[b[:, 0] == l1])


@pytest.mark.parametrize("tag", ["d16", "d32"])
def test_reference_reproduces_fixture(tag):
    O = _oracle()
    if not os.path.isfile(O.ref_amr_path()):
        pytest.skip("reference not compiled here")
    d = np.load(FIXTURE)
    dom, mx, nd, nr = d[f"params_{tag}"]
    got = O.amr_levels_reference(d["x"], d["y"], d["z"], int(dom), int(mx), float(nd), float(nr))
    assert np.array_equal(got, d[f"levels_{tag}"])


def test_domain_density_restatement_matches_fixture():
    O = _oracle()
    d = np.load(FIXTURE)
    got = O.domain_dens_oracle(d["x"], d["y"], d["z"], 16)
    assert np.array_equal(got, d["dens_d16"])
    # every particle is spread over 27 nodes with weights summing to one:
    # the grid's mean density contrast is zero up to the float sums
    assert abs(got.mean()) < 1e-4


@pytest.mark.parametrize("l1", [8, 32, 64])
def test_domain_density_restatement_matches_reference_live(l1):
    O = _oracle()
    if not os.path.isfile(O.ref_amr_path()):
        pytest.skip("reference not compiled here")
    rng = np.random.default_rng(l1)
    n = 20000
    p = rng.random((3, n)).astype(np.float32)
    p[:, :10] = 0.0
    p[0, 10:20] = np.float32(1 - 2 ** -24)
    p[1, 20:30] = 1.0                                   # folded into cell 0, as the reference does
    p[:, 30:40] = np.float32(0.5) / l1                  # exactly on node centres
    p[:, 40:50] = np.float32(1.0) / l1                  # exactly on cell faces
    p[:, 1000:3000] = (0.3 + 0.02 * rng.standard_normal((3, 2000))).astype(np.float32) % np.float32(1.0)
    a = O.domain_dens_oracle(p[0], p[1], p[2], l1)
    b = O.domain_dens_reference(p[0], p[1], p[2], l1)
    assert np.array_equal(a, b)


def test_first_refinement_restatement_matches_fixture():
    O = _oracle()
    d = np.load(FIXTURE)
    got = O.first_refinement_oracle(d["x"], d["y"], d["z"], 32, 5.0)
    assert np.array_equal(got, d["first_ref_d32"].astype(np.int64))
    assert len(got) % 8 == 0                            # whole 2x2x2 blocks of fine nodes


def _first_ref_cases():
    rng = np.random.default_rng(5)
    p = rng.random((3, 30000)).astype(np.float32)
    p[:, :15000] = (0.97 + 0.03 * rng.standard_normal((3, 15000))).astype(np.float32) % np.float32(1.0)
    yield "cluster across the periodic corner", p, 32
    p = rng.random((3, 30000)).astype(np.float32)
    yield "dense: the whole grid refines", p, 16
    p = rng.random((3, 3000)).astype(np.float32)
    p[:, :60] = (0.5 + 0.001 * rng.standard_normal((3, 60))).astype(np.float32)
    yield "one small clump", p, 32
    yield "nothing refines", rng.random((3, 3000)).astype(np.float32), 32


def test_first_refinement_restatement_matches_reference_live():
    O = _oracle()
    if not os.path.isfile(O.ref_amr_path()):
        pytest.skip("reference not compiled here")
    for name, p, l1 in _first_ref_cases():
        ref = O.first_refinement_reference(p[0], p[1], p[2], l1, 5.0, 5.0)
        got = O.first_refinement_oracle(p[0], p[1], p[2], l1, 5.0)
        assert np.array_equal(got, ref), name


def _digest(zyx, dens):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import amr_digest
    return amr_digest(zyx, dens)


@pytest.mark.parametrize("tag", ["d16", "d32"])
def test_hierarchy_restatement_matches_fixture_counts(tag):
    O = _oracle()
    d = np.load(FIXTURE)
    dom, mx, nd, nr = d[f"params_{tag}"]
    got = O.amr_levels_oracle(d["x"], d["y"], d["z"], int(dom), int(mx), float(nd), float(nr))
    assert np.array_equal(got, d[f"levels_{tag}"])


def test_hierarchy_restatement_matches_fixture_every_grid():
    """Nodes (in order) and float densities of all nine grids, 16^3 to 4096^3."""
    O = _oracle()
    d = np.load(FIXTURE)
    want = d["level_digest_d16"]
    for lev in range(len(want)):
        zyx, dens = O.amr_nodes_oracle(d["x"], d["y"], d["z"], 16, 4096, 5.0, 5.0, lev)
        assert _digest(zyx, dens) == int(want[lev]), lev
        key = (zyx[:, 0] * 8192 + zyx[:, 1]) * 8192 + zyx[:, 2]
        assert np.all(np.diff(key) > 0), lev            # the reference's node order is ascending (z, y, x)


def test_hierarchy_restatement_matches_reference_live():
    """Three clusters, two across periodic faces: every grid equal."""
    O = _oracle()
    if not os.path.isfile(O.ref_amr_path()):
        pytest.skip("reference not compiled here")
    rng = np.random.default_rng(11)
    n = 40000
    p = rng.random((3, n)).astype(np.float32)
    for k, c in enumerate([(0.98, 0.01, 0.5), (0.5, 0.99, 0.02), (0.3, 0.3, 0.3)]):
        m = slice(k * 8000, (k + 1) * 8000)
        p[:, m] = ((np.array(c)[:, None] + 0.01 * rng.standard_normal((3, 8000)) * (1 + rng.random(8000)))
                   % 1.0).astype(np.float32)
    lv = O.amr_levels_reference(p[0], p[1], p[2], 32, 2048, 5.0, 5.0)
    assert len(lv) >= 4
    assert np.array_equal(O.amr_levels_oracle(p[0], p[1], p[2], 32, 2048, 5.0, 5.0), lv)
    for lev in range(len(lv)):
        a = O.amr_nodes_oracle(p[0], p[1], p[2], 32, 2048, 5.0, 5.0, lev)
        b = O.amr_nodes_reference(p[0], p[1], p[2], 32, 2048, 5.0, 5.0, lev)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), lev


def test_particle_lists_are_in_index_order_by_level():
    """ll prepends in index order and relink reverses the particles it
    moves, so on every grid each node's list is in index order, descending
    on even grids and ascending on odd ones: a node's density is then a sum
    over its source nodes in node order, each in index order, which a GPU
    gather can reproduce exactly."""
    O = _oracle()
    d = np.load(FIXTURE)
    assert O.amr_list_order_violations(d["x"], d["y"], d["z"], 16, 4096, 5.0, 5.0) == 0


def test_densities_as_a_gather_equal_the_scatter():
    """The formulation a GPU kernel can use without atomics — each node sums
    its source nodes in node order, each source's particles in list order —
    gives every grid's float densities bit for bit."""
    O = _oracle()
    d = np.load(FIXTURE)
    assert O.amr_gather_mismatches(d["x"], d["y"], d["z"], 16, 4096, 5.0, 5.0) == 0
