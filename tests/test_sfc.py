"""Hilbert keys and the particle sort by key (src/main.c:342-356, libsfc).

CPU: the restated key (oracle/ahf_oracle.c, ahforacle_sfc_key) equal to the
reference's own sfc_curve_calcKey (compiled unchanged into oracle/_ref) for
every level count 1..21 and at the box edges; hand-worked first-level order;
the Hilbert property (consecutive keys are face-adjacent cells) over every
cell at 2 and 3 levels; the sort equal to the reference's qsort (keys, and
each run of equal keys as a set; live and the committed fixture
tests/golden/sfc_cfg1.npz).  GPU: ahfgpu_sfc_sort_device equal to the
restatement, keys and order (equal keys by original index).
Bar: identical integers.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle
    oracle.build()
    return oracle


def _key_fn(O):
    import ctypes as C
    lib = C.CDLL(O.oracle_path())
    fn = lib.ahforacle_sfc_key
    fn.argtypes = [C.c_double, C.c_double, C.c_double, C.c_uint]
    fn.restype = C.c_uint64
    return fn


def test_first_level_hand_order():
    """One level: the key is the Gray decode of the octant bits (c0, c1, c2)."""
    O = _oracle()
    key = _key_fn(O)
    want = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3,
            (0, 1, 1): 4, (1, 1, 1): 5, (1, 0, 1): 6, (0, 0, 1): 7}
    for (a, b, c), k in want.items():
        assert key(0.25 + 0.5 * a, 0.25 + 0.5 * b, 0.25 + 0.5 * c, 1) == k


@pytest.mark.parametrize("bits", [2, 3])
def test_keys_walk_face_adjacent_cells(bits):
    O = _oracle()
    key = _key_fn(O)
    m = 1 << bits
    cells = {}
    for i in range(m):
        for j in range(m):
            for k in range(m):
                kk = key((i + 0.5) / m, (j + 0.5) / m, (k + 0.5) / m, bits)
                cells[kk] = (i, j, k)
    assert sorted(cells) == list(range(m ** 3))
    for kk in range(1, m ** 3):
        a, b = np.array(cells[kk - 1]), np.array(cells[kk])
        assert np.abs(a - b).sum() == 1


def test_keys_match_reference_all_levels():
    O = _oracle()
    if not O.have_ref():
        pytest.skip("reference not compiled here")
    key = _key_fn(O)
    rng = np.random.default_rng(3)
    edge = [0.0, 1.0, float(np.float32(1 - 2 ** -24)), 0.5, 0.25, 0.75, 1e-7]
    for bits in range(1, 22):
        pts = [tuple(rng.random(3)) for _ in range(300)] + [(a, b, c) for a in edge for b in edge[:3] for c in edge[:2]]
        for x, y, z in pts:
            assert key(x, y, z, bits) == O.sfc_key_reference(x, y, z, bits), (bits, x, y, z)


def _points(n, seed, ties):
    rng = np.random.default_rng(seed)
    p = rng.random((3, n)).astype(np.float32)
    p[:, :20] = 0.0
    p[0, 20:30] = np.float32(1 - 2 ** -24)
    p[:, 30:40] = 1.0                                   # capped to the last cell
    if ties:                                            # repeated positions and shared finest cells
        p[:, 100:300] = p[:, 40:240]
        p[:, 400:500] = np.float32(0.123456)
    return p


@pytest.mark.parametrize("ties", [False, True])
def test_sort_matches_reference(ties):
    O = _oracle()
    if not O.have_ref():
        pytest.skip("reference not compiled here")
    x, y, z = _points(100000, 5, ties)
    k1, o1 = O.sfc_sort_oracle(x, y, z)
    k2, o2 = O.sfc_sort_reference(x, y, z)
    assert np.array_equal(k1, k2)
    starts = np.flatnonzero(np.r_[True, k1[1:] != k1[:-1]])
    ends = np.r_[starts[1:], len(k1)]
    for s, e in zip(starts, ends):
        if e - s > 1:
            assert sorted(o1[s:e]) == sorted(o2[s:e])
        else:
            assert o1[s] == o2[s]
    assert np.all(np.diff(o1.astype(np.int64))[k1[1:] == k1[:-1]] > 0)   # equal keys by original index


def test_sort_matches_reference_fixture():
    """tests/golden/sfc_cfg1.npz: the reference's own keys and qsort order on
    a cfg1 snapshot with edge and repeated positions (make_golden.py)."""
    O = _oracle()
    d = np.load(os.path.join(HERE, "golden", "sfc_cfg1.npz"))
    k, o = O.sfc_sort_oracle(d["x"], d["y"], d["z"])
    assert np.array_equal(k, d["keys"])
    same = np.r_[False, k[1:] == k[:-1]]
    assert same.any()                                   # the fixture holds equal keys
    assert np.array_equal(o[~same & ~np.r_[same[1:], False]], d["order"][~same & ~np.r_[same[1:], False]])
    starts = np.flatnonzero(~same)
    for s_, e_ in zip(starts, np.r_[starts[1:], len(k)]):
        assert sorted(o[s_:e_]) == sorted(d["order"][s_:e_])


HARNESS = r"""
#include <cstdio>
#include <vector>
#include "sfc_key.cuh"
int main(int argc, char** argv) {
  FILE* f = std::fopen(argv[1], "rb");
  unsigned long long n; int bits;
  if (std::fread(&n, 8, 1, f) != 1 || std::fread(&bits, 4, 1, f) != 1) return 1;
  std::vector<float> p(3 * n);
  if (std::fread(p.data(), 4, 3 * n, f) != 3 * n) return 1;
  std::fclose(f);
  std::vector<unsigned long long> k(n);
  for (unsigned long long i = 0; i < n; i++) k[i] = ahfgpu::hilbert_key(p[3 * i], p[3 * i + 1], p[3 * i + 2], bits);
  FILE* g = std::fopen(argv[2], "wb");
  std::fwrite(k.data(), 8, n, g);
  std::fclose(g);
  return 0;
}
"""


def test_kernel_key_function_host_compiled_matches_oracle(tmp_path):
    """The level loop the sort kernel runs (ahf_gb300/csrc/sfc_key.cuh),
    compiled as host code, equal to the restatement (itself pinned to the
    reference above) for float positions at every level count."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    O = _oracle()
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(os.path.dirname(HERE), "ahf_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    key = _key_fn(O)
    pts = _points(3000, 7, True).T.copy()
    for bits in (1, 2, 3, 7, 13, 20, 21):
        inp = tmp_path / "in.bin"
        with open(inp, "wb") as f:
            f.write(np.uint64(len(pts)).tobytes() + np.int32(bits).tobytes() + pts.astype(np.float32).tobytes())
        subprocess.run([str(exe), str(inp), str(tmp_path / "out.bin")], check=True)
        got = np.fromfile(tmp_path / "out.bin", dtype=np.uint64)
        want = np.array([key(float(a), float(b), float(c), bits) for a, b, c in pts], dtype=np.uint64)
        assert np.array_equal(got, want), bits


@pytest.mark.gpu
@pytest.mark.parametrize("n,ties", [(1, False), (1000, True), (3_000_000, True)])
def test_gpu_sfc_sort_matches_restatement(n, ties):
    import torch
    from ahf_gb300 import build, lib
    build.build()
    lib.init(0)
    O = _oracle()
    if n >= 40 * 1000:
        x, y, z = _points(n, 9, ties)
    else:
        x, y, z = np.random.default_rng(n).random((3, n)).astype(np.float32)
        if ties and n > 10:
            x[n // 2:], y[n // 2:], z[n // 2:] = x[:n - n // 2], y[:n - n // 2], z[:n - n // 2]
    k1, o1 = O.sfc_sort_oracle(x, y, z)
    t = [torch.as_tensor(v).cuda() for v in (x, y, z)]
    keys, order = lib.sfc_sort_device(*t)
    assert np.array_equal(keys.cpu().numpy().view(np.uint64), k1)
    assert np.array_equal(order.cpu().numpy().astype(np.uint64), o1)
