"""Build of the in-tree CUDA library ahf_gb300/libahfgpu.so (sm_103a only).

Each translation unit is compiled by nvcc in parallel and linked into one
shared library with the CUDA runtime linked statically, so the library only
needs the CUDA driver at run time.  The stage's units (halo_fp64.cu,
fp32c_*.cu, amr*.cu) are compiled with --fmad=false: their FP64 paths must round like
the reference's C build, and the float-float arithmetic needs its products
and sums unfused.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libahfgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]
UNITS = {
    "api.cu": [],
    "halo_fp64.cu": ["--fmad=false"],
    "fp32c_class0.cu": ["--fmad=false"],
    "fp32c_class1.cu": ["--fmad=false"],
    "fp32c_class2.cu": ["--fmad=false"],
    "fp32c_finish.cu": ["--fmad=false"],
    "fp32c_small.cu": ["--fmad=false"],
    "fp32c_dispatch.cu": [],
    "noalloc.cu": [],
    "gather.cu": [],
    "writer.cu": [],
    "sfc.cu": [],
    "shard.cu": [],
    "amr.cu": ["--fmad=false"],
    "amr_tree.cu": ["--fmad=false"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build(force: bool = False, verbose: bool = False, defines: tuple = (), out: str | None = None) -> str:
    """Compile every unit and link LIB (or `out`, with extra -D `defines`)."""
    if defines or out:
        return _build_variant(list(defines), out or LIB, verbose)
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def _build_variant(defines, out, verbose):
    bdir = os.path.join(os.path.dirname(os.path.abspath(out)), "_build_variant")
    os.makedirs(bdir, exist_ok=True)
    objs = []
    for src, extra in UNITS.items():
        obj = os.path.join(bdir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc(), *ARCH, *COMMON, *extra, *[f"-D{d}" for d in defines], "-c", os.path.join(CSRC, src), "-o", obj]
        objs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=len(objs)) as ex:
        res = list(ex.map(lambda c: subprocess.run(c[0], capture_output=True, text=True), objs))
    for r in res:
        if r.returncode != 0:
            raise RuntimeError(r.stderr)
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", out, *[o for _, o in objs], "-cudart", "static"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return out


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
