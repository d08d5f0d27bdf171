"""Failure handling at the boundary: an allocation that fails returns a status.

AHF's own code calls exit() when an allocation fails (ahf_halos_sfc.c:339-344);
the library instead returns a negative AHFGPU_ERR_* code and stays usable, and
the caller decides (the shim maps it to common_terminate).  The failures are
made on the host, with no GPU fault: AHFGPU_INJECT_OOM names the allocation
site whose allocations fail as real ones would --
  device_work  the cudaMalloc of the call's work space,
  host_result  the result's page-locked block and its malloc fallback,
  host_plan    a host container of the call's plan (std::bad_alloc, which the
               library catches before it can cross the C ABI).
Each case checks the status and the message, then that the next call without
the injection gives the same result as before.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    from ahf_gb300 import abi, build, lib, synth
    build.build()
    lib.init(0)
    L = synth.generate("cfg3", scale=0.002, max_particles=20000)
    params = synth.params_for(L)
    want = lib.construct_halos(params, L, "batched_fp32c")
    return lib, abi, params, L, want


def _same(a, b):
    return np.array_equal(a.member_off, b.member_off) and np.array_equal(a.member, b.member) and \
        np.array_equal(a.halo["M_vir"], b.halo["M_vir"])


@pytest.mark.parametrize("site", ["host_plan", "host_result"])
def test_injected_host_allocation_failure_returns_oom(case, monkeypatch, site):
    lib, abi, params, L, want = case
    monkeypatch.setenv("AHFGPU_INJECT_OOM", site)
    with pytest.raises(lib.AhfGpuError) as e:
        lib.construct_halos(params, L, "batched_fp32c")
    assert e.value.code == abi.AHFGPU_ERR_OOM
    assert "alloc" in str(e.value)
    monkeypatch.delenv("AHFGPU_INJECT_OOM")
    assert _same(lib.construct_halos(params, L, "batched_fp32c"), want)


def test_injected_device_allocation_failure_returns_oom(case, monkeypatch):
    lib, abi, params, L, want = case
    # a fresh context holds no work space, so the next call must allocate it
    lib.shutdown()
    lib.init(0)
    monkeypatch.setenv("AHFGPU_INJECT_OOM", "device_work")
    with pytest.raises(lib.AhfGpuError) as e:
        lib.construct_halos(params, L, "batched_fp64")
    assert e.value.code == abi.AHFGPU_ERR_OOM
    assert "cudaMalloc" in str(e.value)
    monkeypatch.delenv("AHFGPU_INJECT_OOM")
    got = lib.construct_halos(params, L, "batched_fp64")
    assert np.array_equal(got.member, want.member)


def test_invalid_offsets_return_invalid_without_abort(case):
    lib, abi, params, L, want = case
    bad = L.select(np.arange(L.nhalo))
    bad.off = bad.off.copy()
    bad.off[3], bad.off[4] = bad.off[4], bad.off[3]   # not monotone
    with pytest.raises(lib.AhfGpuError) as e:
        lib.construct_halos(params, bad, "batched_fp32c")
    assert e.value.code == abi.AHFGPU_ERR_INVALID
    assert _same(lib.construct_halos(params, L, "batched_fp32c"), want)
