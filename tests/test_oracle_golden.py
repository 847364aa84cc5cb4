"""The CPU oracle against the reference program's own outputs.

Each fixture holds what the reference (main_3d.cu, built with its one compile
fix, run on a GB300) produced for a seeded synthetic case: digests of its
eight pairing arrays, its corrected field, edit counters, iteration count and
the delta buffer of its first fix round.  These tests pin the oracle; the GPU
tests then compare the product with the oracle.
"""
import os

import numpy as np
import pytest

from conftest import fixture_files, load_fixture, reference_cnt, reference_fixed, sha
from oracle import oracle as O

FIXTURES = fixture_files()


def _id(p):
    return os.path.basename(p)[4:-4]


def test_fixtures_present():
    assert len(FIXTURES) >= 10


@pytest.mark.parametrize("path", FIXTURES, ids=_id)
def test_inputs_regenerate(path):
    meta, z, f, g = load_fixture(path)
    assert sha(f) == str(z["f_sha"]) and sha(g) == str(z["g_sha"])


@pytest.mark.parametrize("path", FIXTURES, ids=_id)
def test_oracle_pairing_matches_reference(path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    P = O.pair(f, dims, threads=4)
    for a, k in zip(P, ("PV", "PE", "PF", "PT")):
        assert sha(a) == meta[k + "_sha256"], k
        assert int((a == -1).sum()) == meta[k + "_ncrit"]
    if meta["flags"][3] == 0:  # with filtration the reference pairs the filtered field
        Q = O.pair(g, dims, threads=4)
        for a, k in zip(Q, ("QV", "QE", "QF", "QT")):
            assert sha(a) == meta[k + "_sha256"], k


@pytest.mark.parametrize("path", FIXTURES, ids=_id)
def test_oracle_correction_matches_reference(path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    out, st, cnt = O.correct(f, g, dims, meta["rel"], meta["flags"], max_outer=1000, threads=4)
    assert st["converged"] and st["oob"] == 0
    ref = reference_fixed(z, g)
    assert sha(ref) == str(z["fixed_sha"])
    assert np.array_equal(out, ref), f"{int((out != ref).sum())} values differ"
    assert np.array_equal(cnt, reference_cnt(z, f.size))
    # the reference prints total_ite + 1 as "iteration number"
    assert st["outer_iterations"] + 1 == meta["iteration_number"]


@pytest.mark.parametrize("path", [p for p in FIXTURES if "1001000" not in p], ids=_id)
def test_oracle_first_fix_round_matches_reference(path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    P = O.pair(f, dims, threads=4)
    Q = O.pair(g, dims, threads=4)
    lists = O.cp_mismatch(P, Q, dims)
    rng = float(f.max() - f.min())
    bound = rng * meta["rel"]
    cnt = np.ones(f.size, np.int32)
    buf, oob = O.fix_cp(f, g, cnt, bound, rng, meta["flags"][6], meta["flags"][0], P, Q, lists, dims)
    assert oob == 0
    idx = np.nonzero(buf != -2000.0 * rng)[0]
    assert np.array_equal(idx, z["r0_idx"])
    assert np.array_equal(buf[idx], z["r0_buf"])


def test_oracle_euler_characteristic():
    """#min - #1-saddle + #2-saddle - #max = 1 for a box."""
    from dmtz_gb300 import synth

    for dims in ((5, 6, 7), (9, 4, 3), (2, 2, 2)):
        f = synth.power_law(dims, 3).reshape(-1)
        P = O.pair(f, dims)
        c = [int((a == -1).sum()) for a in P]
        assert c[0] - c[1] + c[2] - c[3] == 1
