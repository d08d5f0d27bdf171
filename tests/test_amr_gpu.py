"""The AMR hierarchy on the GPU, against the oracle and the reference's own
output.

ahfgpu_amr_domain_density_device replaces gen_domgrids + ll + assign_npart
for the domain grid (src/libamr_serial/generate_grids.c:24, density.c:238):
its float densities must equal, bit for bit, the oracle's restatement
(ahforacle_domain_dens, pinned against the reference) and the reference's own
floats in tests/golden/amr_cfg1.npz (dens_d16).
ahfgpu_amr_first_refinement_device replaces the first refine_grid call
(refine_grid.c:899): the fine nodes must equal the oracle's
(ahforacle_first_refinement) and, as a set, the reference's own first refined
grid in the fixture (first_ref_d32, in the reference's quad order).
ahfgpu_amr_hierarchy_device replaces the whole grid generation
(src/main.c:614-648, gen_AMRhierarchy, generate_grids.c:278): every grid's
nodes per dimension, node count and listed particles must equal the
reference's own (levels_d16 / levels_d32 in the fixture) and the oracle's,
and every grid's nodes (in order) and float densities the oracle's
restatement bit for bit and the reference's own grids through their
digests (level_digest_d16).
Inputs: the cfg1 snapshot of the fixture, seeded uniform points with
coordinates exactly 0, 1 - 2^-24 and 1.0 (folded into node 0), odd grid
sizes, clusters across periodic faces, and the 64^3 and 256^3-particle
cfg1 and cfg2 boxes.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "amr_cfg1.npz")


@pytest.fixture(scope="module")
def gpu():
    from ahf_gb300 import build, lib
    build.build()
    lib.init(0)
    return lib


def _dev(*a):
    import torch
    return [torch.as_tensor(np.ascontiguousarray(v, np.float32)).cuda() for v in a]


def _edge_points(n, seed):
    rng = np.random.default_rng(seed)
    x, y, z = (rng.random(n).astype(np.float32) for _ in range(3))
    x[:5], y[5:9], z[9:12] = 0.0, np.float32(1 - 2 ** -24), 1.0
    x[12:14], y[12:14], z[12:14] = 1.0, 1.0, 1.0
    return x, y, z


@pytest.mark.parametrize("l1", [16, 32, 64])
def test_domain_density_equals_oracle_on_cfg1(gpu, oracle_built, l1):
    d = np.load(FIXTURE)
    x, y, z = d["x"], d["y"], d["z"]
    got = gpu.amr_domain_density_device(*_dev(x, y, z), l1).cpu().numpy()
    want = oracle_built.domain_dens_oracle(x, y, z, l1).ravel()
    assert np.array_equal(got.astype(np.float64), want)


@pytest.mark.parametrize("l1,n", [(3, 200), (5, 3000), (8, 20000), (17, 50000)])
def test_domain_density_equals_oracle_with_edges(gpu, oracle_built, l1, n):
    x, y, z = _edge_points(n, seed=l1)
    got = gpu.amr_domain_density_device(*_dev(x, y, z), l1).cpu().numpy()
    want = oracle_built.domain_dens_oracle(x, y, z, l1).ravel()
    assert np.array_equal(got.astype(np.float64), want)


def test_domain_density_equals_reference_fixture(gpu):
    d = np.load(FIXTURE)
    got = gpu.amr_domain_density_device(*_dev(d["x"], d["y"], d["z"]), 16).cpu().numpy()
    assert np.array_equal(got.astype(np.float64), np.asarray(d["dens_d16"], np.float64).ravel())


def test_first_refinement_equals_oracle_and_reference(gpu, oracle_built):
    d = np.load(FIXTURE)
    x, y, z = d["x"], d["y"], d["z"]
    dens = gpu.amr_domain_density_device(*_dev(x, y, z), 32)
    got = gpu.amr_first_refinement_device(dens, 32, len(x), 5.0).cpu().numpy().astype(np.int64)
    want = oracle_built.first_refinement_oracle(x, y, z, 32, 5.0)
    assert len(got) > 0
    assert np.array_equal(got, np.asarray(want, np.int64).reshape(-1, 3))
    ref = np.asarray(d["first_ref_d32"], np.int64).reshape(-1, 3)
    key = lambda a: np.sort((a[:, 0] * 4096 + a[:, 1]) * 4096 + a[:, 2])
    assert np.array_equal(key(got), key(ref))


@pytest.mark.parametrize("nth", [1.0, 3.0, 40.0, 1e9])
def test_first_refinement_thresholds(gpu, oracle_built, nth):
    x, y, z = _edge_points(30000, seed=7)
    x[:3000] = (0.3 + 0.01 * np.random.default_rng(1).random(3000)).astype(np.float32)   # a dense clump
    dens = gpu.amr_domain_density_device(*_dev(x, y, z), 24)
    got = gpu.amr_first_refinement_device(dens, 24, len(x), nth).cpu().numpy().astype(np.int64)
    want = np.asarray(oracle_built.first_refinement_oracle(x, y, z, 24, nth), np.int64).reshape(-1, 3)
    assert np.array_equal(got, want)   # 1e9: nothing flagged, no fine grid (MIN_NNODES)


@pytest.mark.slow
def test_domain_density_cfg2_box(gpu, oracle_built):
    from ahf_gb300 import synth
    S = synth.box_snapshot("cfg2")
    p = (S.pos / np.float32(S.box)).astype(np.float32)
    x, y, z = (np.ascontiguousarray(p[:, k]) for k in range(3))
    dens = gpu.amr_domain_density_device(*_dev(x, y, z), 64)
    assert np.array_equal(dens.cpu().numpy().astype(np.float64), oracle_built.domain_dens_oracle(x, y, z, 64).ravel())
    got = gpu.amr_first_refinement_device(dens, 64, len(x), 5.0).cpu().numpy().astype(np.int64)
    want = np.asarray(oracle_built.first_refinement_oracle(x, y, z, 64, 5.0), np.int64).reshape(-1, 3)
    assert np.array_equal(got, want)


def test_invalid_grid_is_rejected(gpu):
    from ahf_gb300 import abi
    x, y, z = _dev(*_edge_points(100, seed=2))
    with pytest.raises(gpu.AhfGpuError) as e:
        gpu.amr_domain_density_device(x, y, z, 2)
    assert e.value.code == abi.AHFGPU_ERR_INVALID


def _hier_same_as_oracle(gpu, O, x, y, z, dom, mx, nd, nr):
    lv = gpu.amr_hierarchy_device(*_dev(x, y, z), dom, mx, nd, nr)
    want = O.amr_levels_oracle(x, y, z, dom, mx, nd, nr)
    assert np.array_equal(lv, want)
    for g in range(len(lv)):
        zyx, dens = gpu.amr_grid_device(g)
        a = O.amr_nodes_oracle(x, y, z, dom, mx, nd, nr, g)
        assert np.array_equal(zyx.cpu().numpy().astype(np.int64), a[0]), g
        assert np.array_equal(dens.cpu().numpy().astype(np.float64), a[1]), g
    return lv


@pytest.mark.parametrize("tag", ["d16", "d32"])
def test_hierarchy_equals_reference_fixture(gpu, tag):
    d = np.load(FIXTURE)
    dom, mx, nd, nr = d[f"params_{tag}"]
    lv = gpu.amr_hierarchy_device(*_dev(d["x"], d["y"], d["z"]), int(dom), int(mx), float(nd), float(nr))
    assert np.array_equal(lv, d[f"levels_{tag}"])
    if tag == "d16":   # nodes and densities of all nine grids, 16^3 to 4096^3
        import sys
        sys.path.insert(0, os.path.join(HERE, "golden"))
        from make_golden import amr_digest
        for g, want in enumerate(d["level_digest_d16"]):
            zyx, dens = gpu.amr_grid_device(g)
            assert amr_digest(zyx.cpu().numpy().astype(np.int64), dens.cpu().numpy().astype(np.float64)) == int(want), g


def test_hierarchy_equals_oracle_on_cfg1(gpu, oracle_built):
    d = np.load(FIXTURE)
    lv = _hier_same_as_oracle(gpu, oracle_built, d["x"], d["y"], d["z"], 16, 4096, 5.0, 5.0)
    assert len(lv) == 9


def _clusters(seed=11, n=40000):
    rng = np.random.default_rng(seed)
    p = rng.random((3, n)).astype(np.float32)
    for k, c in enumerate([(0.98, 0.01, 0.5), (0.5, 0.99, 0.02), (0.3, 0.3, 0.3)]):
        m = slice(k * 8000, (k + 1) * 8000)
        p[:, m] = ((np.array(c)[:, None] + 0.01 * rng.standard_normal((3, 8000)) * (1 + rng.random(8000)))
                   % 1.0).astype(np.float32)
    return p


@pytest.mark.parametrize("dom,mx,nd,nr", [(32, 2048, 5.0, 5.0), (8, 4096, 2.0, 3.0), (9, 576, 5.0, 5.0)])
def test_hierarchy_clusters_across_faces(gpu, oracle_built, dom, mx, nd, nr):
    p = _clusters()
    lv = _hier_same_as_oracle(gpu, oracle_built, p[0], p[1], p[2], dom, mx, nd, nr)
    assert len(lv) >= 3


def test_hierarchy_uniform_with_edges_odd_domain(gpu, oracle_built):
    x, y, z = _edge_points(20000, seed=5)
    _hier_same_as_oracle(gpu, oracle_built, x, y, z, 5, 640, 1.0, 1.0)


def test_hierarchy_stops_without_refinement(gpu, oracle_built):
    x, y, z = _edge_points(3000, seed=3)
    lv = _hier_same_as_oracle(gpu, oracle_built, x, y, z, 16, 1024, 1e9, 5.0)
    assert len(lv) == 1                     # nothing above the threshold: the domain grid only
    lv = _hier_same_as_oracle(gpu, oracle_built, x, y, z, 16, 16, 5.0, 5.0)
    assert len(lv) == 1                     # ngrid_max reached


@pytest.mark.slow
@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_hierarchy_box(gpu, oracle_built, name):
    from ahf_gb300 import synth
    S = synth.box_snapshot(name)
    p = (S.pos / np.float32(S.box)).astype(np.float32)
    x, y, z = (np.ascontiguousarray(p[:, k]) for k in range(3))
    lv = gpu.amr_hierarchy_device(*_dev(x, y, z), 64, 16384, 5.0, 5.0)
    assert np.array_equal(lv, oracle_built.amr_levels_oracle(x, y, z, 64, 16384, 5.0, 5.0))
    assert len(lv) >= 7
    for g, (zyx_o, dens_o) in enumerate(oracle_built.amr_all_nodes_oracle(x, y, z, 64, 16384, 5.0, 5.0)):
        zyx, dens = gpu.amr_grid_device(g)
        assert np.array_equal(zyx.cpu().numpy().astype(np.int64), zyx_o), g
        assert np.array_equal(dens.cpu().numpy().astype(np.float64), dens_o), g


def test_hierarchy_invalid_arguments(gpu):
    from ahf_gb300 import abi
    x, y, z = _dev(*_edge_points(100, seed=2))
    with pytest.raises(gpu.AhfGpuError) as e:
        gpu.amr_hierarchy_device(x, y, z, 16, 8, 5.0, 5.0)      # ngrid_max below the domain grid
    assert e.value.code == abi.AHFGPU_ERR_INVALID
    with pytest.raises(gpu.AhfGpuError) as e:
        gpu.amr_grid_device(99)
    assert e.value.code == abi.AHFGPU_ERR_INVALID
