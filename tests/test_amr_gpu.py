"""The AMR hierarchy's first two levels on the GPU, against the oracle and
the reference's own output.

ahfgpu_amr_domain_density_device replaces gen_domgrids + ll + assign_npart
for the domain grid (src/libamr_serial/generate_grids.c:24, density.c:238):
its float densities must equal, bit for bit, the oracle's restatement
(ahforacle_domain_dens, pinned against the reference) and the reference's own
floats in tests/golden/amr_cfg1.npz (dens_d16).
ahfgpu_amr_first_refinement_device replaces the first refine_grid call
(refine_grid.c:899): the fine nodes must equal the oracle's
(ahforacle_first_refinement) and, as a set, the reference's own first refined
grid in the fixture (first_ref_d32, in the reference's quad order).
Inputs: the cfg1 snapshot of the fixture, seeded uniform points with
coordinates exactly 0, 1 - 2^-24 and 1.0 (folded into node 0), odd grid
sizes, and the 256^3-particle cfg2 box.
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
