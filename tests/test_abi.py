"""Host-side checks of the C ABI (no GPU needed): the library loads, exports
every entry point include/ahfgpu.h declares, the ctypes mirror has the C
layout, and calls fail cleanly with status codes instead of aborting."""
import ctypes as C
import os
import re
import subprocess

import pytest

from ahf_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ahfgpu.h")


@pytest.fixture(scope="module")
def libpath():
    from ahf_gb300 import build
    return build.build()


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"AHFGPU_API\s+[\w\s\*]*?\b(ahfgpu_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("ahfgpu_init", "ahfgpu_construct_halos", "ahfgpu_construct_halos_device", "ahfgpu_result_free",
              "ahfgpu_last_error", "ahfgpu_version", "ahfgpu_shutdown", "ahfgpu_fetch_result"):
        assert s in syms


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    lib = C.CDLL(libpath)
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_ctypes_layout_matches_c(tmp_path):
    src = tmp_path / "layout.c"
    checks = {
        "ahfgpu_params": [f[0] for f in abi.Params._fields_],
        "ahfgpu_batch": [f[0] for f in abi.Batch._fields_],
        "ahfgpu_halo": [("lambda" if f[0] == "lambda_" else f[0]) for f in abi.Halo._fields_],
        "ahfgpu_stats": [f[0] for f in abi.Stats._fields_],
        "ahfgpu_result": [f[0] for f in abi.Result._fields_],
        "ahfgpu_particles": [f[0] for f in abi.Particles._fields_],
        "ahfgpu_centres": [f[0] for f in abi.Centres._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for st, fields in checks.items():
        lines.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fields:
            lines.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    lines.append('printf("NFIELDS %d\\n", AHFGPU_PROF_NFIELDS); return 0;}')
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    types = {"ahfgpu_params": abi.Params, "ahfgpu_batch": abi.Batch, "ahfgpu_halo": abi.Halo,
             "ahfgpu_stats": abi.Stats, "ahfgpu_result": abi.Result, "ahfgpu_particles": abi.Particles,
             "ahfgpu_centres": abi.Centres}
    for st, ty in types.items():
        assert int(got[st]) == C.sizeof(ty), st
        for f in ty._fields_:
            cname = "lambda" if f[0] == "lambda_" else f[0]
            assert int(got[f"{st}.{cname}"]) == getattr(ty, f[0]).offset, (st, f[0])
    assert int(got["NFIELDS"]) == abi.PROF_NFIELDS
    assert abi.HALO_DTYPE.itemsize == C.sizeof(abi.Halo)


@pytest.mark.parametrize("compiler,std", [("gcc", "c99"), ("g++", "c++11")])
def test_header_compiles_strictly(tmp_path, compiler, std):
    """AHF is built with gcc -std=c99: the header must compile there (and in
    C++) without a warning."""
    import shutil
    if not shutil.which(compiler):
        pytest.skip(f"no {compiler}")
    src = tmp_path / "h.c"
    src.write_text('#include "ahfgpu.h"\nint main(void) { ahfgpu_params p; ahfgpu_batch b; ahfgpu_result r; '
                   '(void)p; (void)b; (void)r; return ahfgpu_version() ? 0 : 1; }\n')
    lang = ["-x", "c++"] if compiler == "g++" else []
    subprocess.run([compiler, f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.dirname(HEADER), *lang, "-c", str(src), "-o", str(tmp_path / "h.o")], check=True)


def test_calls_fail_cleanly_without_init(libpath):
    from ahf_gb300 import lib, synth
    L = synth.generate("cfg1", scale=0.1)
    p = synth.params_for(L)
    b, keep = abi.make_batch(L)
    r = abi.Result()
    l = lib.load()
    rc = l.ahfgpu_construct_halos(C.byref(p), C.byref(b), C.byref(r), 1)
    assert rc == abi.AHFGPU_ERR_STATE
    assert "init" in lib.last_error()
    assert l.ahfgpu_version().decode().startswith("ahfgpu")


def test_device_entry_points_refuse_before_init(libpath):
    """Every device entry point returns AHFGPU_ERR_STATE, touching none of
    its arguments, until ahfgpu_init has succeeded."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the library may be initialised)")
    from ahf_gb300 import lib
    l = lib.load()
    out, nb = C.c_void_p(), C.c_uint64()
    calls = {
        "ahfgpu_construct_halos_device": lambda: l.ahfgpu_construct_halos_device(None, None, None, 2, None),
        "ahfgpu_fetch_result": lambda: l.ahfgpu_fetch_result(None),
        "ahfgpu_gather_device": lambda: l.ahfgpu_gather_device(None, None, None, None),
        "ahfgpu_gather_radii_device": lambda: l.ahfgpu_gather_radii_device(5, None, None, None, None, None, 0.1,
                                                                           None, None),
        "ahfgpu_write_particles_device": lambda: l.ahfgpu_write_particles_device(None, None, None, 20,
                                                                                 C.byref(out), C.byref(nb), None),
        "ahfgpu_write_particles_bin_device": lambda: l.ahfgpu_write_particles_bin_device(None, None, 20,
                                                                                         C.byref(out), C.byref(nb),
                                                                                         None),
        "ahfgpu_sfc_sort_device": lambda: l.ahfgpu_sfc_sort_device(10, None, None, None, 21, None, None, None),
        "ahfgpu_tuning": lambda: l.ahfgpu_tuning(None, 0),
    }
    for name, call in calls.items():
        assert call() == abi.AHFGPU_ERR_STATE, name
        assert "init" in lib.last_error(), name


def test_init_without_device_reports_no_device(libpath):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ahf_gb300 import lib
    rc = lib.load().ahfgpu_init(0)
    assert rc == abi.AHFGPU_ERR_NO_DEVICE
    with pytest.raises(lib.AhfGpuError):
        lib.check(rc)
