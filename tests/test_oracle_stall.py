"""The oracle's stall breaking (the checker for the GPU's): a round that
changes no value and no edit counter is a fixed point of the reference's
rules; with break_stalls the oracle resets a growing box around the remaining
mismatches to the original values and goes on.  Runs converge, stay within
the bound, end with the original critical cells, and runs that converge
without breaking are unchanged."""
import numpy as np
import pytest

from oracle import oracle as O

EXTREMA_ONLY = [0] * 7
FULL = [1, 1, 1, 0, 0, 0, 0]


def _case(dims, seed, rel, kind="powerlaw", decomp="sz"):
    from dmtz_gb300 import synth

    f, g = synth.make_case(kind, dims, seed, rel, decomp)
    return f.reshape(-1), g.reshape(-1)


@pytest.mark.parametrize("dims,seed,rel,flags", [((16, 16, 16), 0, 1e-3, EXTREMA_ONLY),
                                                 ((16, 16, 16), 2, 1e-2, EXTREMA_ONLY),
                                                 ((32, 28, 24), 1, 1e-2, FULL)])
def test_oracle_breaking(dims, seed, rel, flags):
    f, g = _case(dims, seed, rel)
    _, st0, _ = O.correct(f, g, dims, rel, flags, max_outer=4)
    assert not st0["converged"] and st0["stall_breaks"] == 0
    out, st, cnt = O.correct(f, g, dims, rel, flags, max_outer=200, break_stalls=True)
    assert st["converged"] and st["stall_breaks"] > 0 and st["oob"] == 0
    bound = (f.max() - f.min()) * rel
    assert np.all(np.abs(out - f) <= bound * (1 + 1e-12))
    P, Q = O.pair(f, dims), O.pair(out, dims)
    L = [len(x) for x in O.cp_mismatch(P, Q, dims)]
    if flags[0] != 1:
        L[1] = L[2] = 0
    assert L == [0, 0, 0, 0]
    if flags[1] == 1:
        at, _, de, _, oob = O.path_detect(P, Q, dims)
        assert oob == 0 and len(at) == 0 and len(de) == 0
    # reset values are the original ones; everything else went the reference's way
    assert np.count_nonzero(out == f) > 0 and np.count_nonzero(out != f) > 0


def test_oracle_breaking_leaves_converging_runs():
    f, g = _case((20, 18, 16), 2, 1e-2, "gauss", "uniform")
    a, sa, ca = O.correct(f, g, (20, 18, 16), 1e-2, FULL, max_outer=500)
    b, sb, cb = O.correct(f, g, (20, 18, 16), 1e-2, FULL, max_outer=500, break_stalls=True)
    assert sa["converged"] and sb["stall_breaks"] == 0
    assert np.array_equal(a, b) and np.array_equal(ca, cb)
