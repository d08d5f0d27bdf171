"""The whole AHF program with the stage swapped for the GPU library.

Two builds of the reference's own sources (oracle/Makefile target `ahf`,
serial): the stock AHF, and AHF-gpu, whose loop at
src/libahf/ahf_halos.c:504-510 calls ahfgpu_shim_construct_halos
(ahf_gb300/integration: the patch and the shim) -- AHF's own reader, AMR
hierarchy, halo finding and gather run unchanged, then one
ahfgpu_construct_halos call, then AHF's own re-hash, sorting and writers.

Both run the same synthetic GADGET-1 snapshot (ngrid^3 equal-mass particles,
NFW haloes plus a uniform background) and the output files are compared:
  plain and batched FP64 forms: AHF_particles, AHF_halos, AHF_profiles and
    AHF_substructure byte for byte (bound id sets bit-exact, and every
    printed property equal);
  FP32C form: AHF_particles and AHF_substructure byte for byte; AHF_halos
    and AHF_profiles field by field, integers equal, every printed number
    within 1e-6 relative or one unit of its last printed digit.
cfg1: 64^3 particles in 50 Mpc/h, 20 haloes; cfg2: 256^3 in 200 Mpc/h,
2,000 haloes with subhaloes (slow).
"""
import os
import subprocess

import numpy as np
import pytest

SUFFIXES = ("AHF_halos", "AHF_particles", "AHF_profiles", "AHF_substructure")


@pytest.fixture(scope="module")
def ahf_bins(oracle_built):
    from ahf_gb300 import build
    build.build()
    try:
        return oracle_built.build_ahf()
    except FileNotFoundError as e:
        pytest.skip(str(e))


def _run(binary, tmp, tag, snap_path, snap, env=None):
    from ahf_gb300 import synth
    prefix = os.path.join(tmp, tag)
    inp = prefix + ".input"
    synth.write_gadget1(snap_path, snap, prefix, inp, write_snapshot=not os.path.exists(snap_path))
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([binary, inp], cwd=tmp, env=e, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, (tag, r.stdout[-2000:], r.stderr[-2000:])
    out = {}
    for suf in SUFFIXES:
        files = [f for f in os.listdir(tmp) if f.startswith(tag + ".") and f.endswith(suf)]
        assert len(files) == 1, (tag, suf, files)
        out[suf] = open(os.path.join(tmp, files[0]), "rb").read()
    return out


def _close_text(a: bytes, b: bytes, rtol: float):
    """Field-by-field comparison of two AHF text tables: integer fields
    equal, numbers within rtol relative or one unit of the last printed
    digit of the expected value.  Returns a list of differences."""
    la, lb = a.decode().splitlines(), b.decode().splitlines()
    if len(la) != len(lb):
        return [f"{len(la)} lines vs {len(lb)}"]
    bad = []
    for i, (x, y) in enumerate(zip(la, lb)):
        if x.startswith("#") or y.startswith("#"):
            if x != y:
                bad.append(f"line {i}: header differs")
            continue
        fx, fy = x.split(), y.split()
        if len(fx) != len(fy):
            bad.append(f"line {i}: {len(fx)} fields vs {len(fy)}")
            continue
        for j, (u, v) in enumerate(zip(fx, fy)):
            if u == v:
                continue
            if "." not in v and "e" not in v.lower():
                bad.append(f"line {i} field {j}: {u} vs {v}")
                continue
            fu, fv = float(u), float(v)
            mant = v.lower().split("e")[0]
            dec = len(mant.split(".")[1]) if "." in mant else 0
            exp = int(v.lower().split("e")[1]) if "e" in v.lower() else 0
            ulp = 10.0 ** (exp - dec)
            if abs(fu - fv) > max(rtol * abs(fv), 1.0001 * ulp):
                bad.append(f"line {i} field {j}: {u} vs {v}")
        if len(bad) > 10:
            break
    return bad


def _case(name, tmp_path, ahf_bins, modes):
    from ahf_gb300 import synth
    stock, gpu = ahf_bins
    snap = synth.box_snapshot(name)
    tmp = str(tmp_path)
    snap_path = os.path.join(tmp, f"snap_{name}")
    want = _run(stock, tmp, "stock", snap_path, snap)
    assert want["AHF_particles"].count(b"\n") > 100
    for mode in modes:
        got = _run(gpu, tmp, f"gpu_{mode}", snap_path, snap, {"AHFGPU_MODE": mode})
        assert got["AHF_particles"] == want["AHF_particles"], f"{name} {mode}: AHF_particles differ"
        assert got["AHF_substructure"] == want["AHF_substructure"], f"{name} {mode}: AHF_substructure differ"
        if mode in ("plain", "batched"):
            for suf in ("AHF_halos", "AHF_profiles"):
                assert got[suf] == want[suf], f"{name} {mode}: {suf} differ: " \
                    f"{_close_text(got[suf], want[suf], 0.0)[:5]}"
        else:
            for suf in ("AHF_halos", "AHF_profiles"):
                bad = _close_text(got[suf], want[suf], 1e-6)
                assert not bad, (name, mode, suf, bad[:5])


@pytest.mark.gpu
def test_dropin_cfg1_all_forms_equal_stock_ahf(tmp_path, ahf_bins):
    _case("cfg1", tmp_path, ahf_bins, ("plain", "batched", "fp32c"))


@pytest.mark.gpu
@pytest.mark.slow
def test_dropin_cfg2_plain_equals_stock_ahf(tmp_path, ahf_bins):
    _case("cfg2", tmp_path, ahf_bins, ("plain",))


def test_close_text_rules():
    a = b"#h\n 1  2.50  3.1e+05\n"
    assert _close_text(a, a, 0.0) == []
    assert _close_text(b"#h\n 1  2.51  3.1e+05\n", a, 0.0) == []          # one unit of the last digit
    assert _close_text(b"#h\n 1  2.52  3.1e+05\n", a, 0.0) != []
    assert _close_text(b"#h\n 2  2.50  3.1e+05\n", a, 0.0) != []          # integers exact
    assert np.isfinite(float("3.1e+05"))
