"""The summation rules of the AMR density gathers, on the host.

ahf_gb300/csrc/amr_sum.cuh sums a node's TSC terms as windows of 32: within
a binade of the float accumulator every step is a two-state map of the
accumulator's parity, and maps compose; a term whose result would leave the
binade takes the exact step.  tests/amr_sum_check.cu runs that rule (the
library's own per-term map, composition and exact step, compiled for the
host) against the reference's sequential float sum (density.c:238's
`dens += ...` on a float) on seeded random sequences with exact ties, zero
terms and binade crossings from -1 through zero; the results must be equal
bit for bit.  The GPU tests check the warp code itself against the oracle
on whole hierarchies.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ahf_gb300", "csrc")


def test_windowed_float_sum_equals_sequential_sum(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.isfile(nvcc):
        pytest.skip("no nvcc")
    exe = tmp_path / "amr_sum_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "amr_sum_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    assert words[0] == "mismatches" and int(words[1]) == 0, r.stdout
    assert int(words[5]) > 0          # exact steps were taken (binade changes)
