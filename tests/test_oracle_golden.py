"""The CPU restatement against the reference's own outputs.

The reference has no test suite and no data; tests/golden/*.npz hold the
reference's outputs (oracle/_ref, built from the unmodified AHF sources by
tests/golden/make_golden.py) on seeded inputs and edge cases.  The
restatement must reproduce them bit for bit, except for the eigenvectors
(own Jacobi solver: equal up to sign, 1e-8).
"""
import glob
import os

import numpy as np
import pytest

from compare import compare
from make_golden import load_case

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("gather_", "writer_", "sfc_", "radii_", "amr_")))   # stage cases only


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_restatement_matches_reference_golden(oracle_built, path):
    params, lists, exp = load_case(path)
    got = oracle_built.run_oracle(params, lists)
    bad = compare(got, exp, rtol=0.0, etol=1e-8)
    # bit-exact except eigen-solver rounding on the axis ratios
    bad = [b for b in bad if not b.startswith("axis") and not b.startswith("profile axis")]
    assert not bad, bad
    e = np.abs(got.halo["axis"] - exp["halo_axis"])
    assert np.all(e <= 1e-12), float(e.max())


def test_golden_covers_edge_cases():
    _, lists, exp = load_case(os.path.join(os.path.dirname(__file__), "golden", "edge_cases.npz"))
    flags = exp["halo_flags"]
    n = np.diff(lists.off.astype(np.int64))
    assert (n == 0).any()                               # empty list
    assert ((n > 0) & (n < 20)).any()                    # below MINPART at input
    assert ((flags & 0x008) & ~(flags & 0x010)).any()    # fell below MINPART while unbinding
    assert (exp["halo_npart"] <= 1).any()                # (nearly) everything unbound
    # a particle at distance exactly 0 from its centre
    zero = False
    for h in range(lists.nhalo):
        sl = slice(int(lists.off[h]), int(lists.off[h + 1]))
        d = ((lists.x[sl] - lists.cx[h]) ** 2 + (lists.y[sl] - lists.cy[h]) ** 2 + (lists.z[sl] - lists.cz[h]) ** 2)
        zero |= bool((d == 0).any())
    assert zero
    # straddling the periodic boundary
    assert ((lists.cx < 0.001) | (lists.cx > 0.999)).any()


def test_restatement_vs_reference_live(oracle_built):
    """Where the reference was built here, compare on a fresh seeded batch."""
    import oracle as O
    from ahf_gb300 import synth
    if not O.have_ref(False):
        pytest.skip("reference harness not built on this machine")
    L = synth.generate("cfg4", scale=0.004)
    p = synth.params_for(L)
    a = O.run_oracle(p, L)
    b = O.run_reference(p, L)
    bad = [x for x in compare(a, b, rtol=0.0, etol=1e-8) if "axis" not in x]
    assert not bad, bad
