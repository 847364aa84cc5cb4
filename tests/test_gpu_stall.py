"""Stall breaking.  A round whose update changes no value and no edit counter
is a fixed point of the reference's rules: its loop repeats that round
forever.  With break_stalls (the default) the values in a box around the
remaining mismatched cells go back to the original values and the loop goes
on.  The result must stay within the bound and carry no mismatch the flags ask
about, and runs that converge under the reference's rules must come out
unchanged."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

EXTREMA_ONLY = (0, 0, 0, 0, 0, 0, 0)
FULL = (1, 1, 1, 0, 0, 0, 0)

# power-law fields with the sparse-error decompression: under extrema-only
# flags the reference's rules reach a fixed point with mismatches left
STALLING = [((16, 16, 16), 0, 1e-3), ((16, 16, 16), 2, 1e-2), ((24, 20, 18), 1, 1e-3), ((24, 20, 18), 3, 1e-2)]


def _case(dims, seed, rel, kind="powerlaw", decomp="sz"):
    from dmtz_gb300 import synth

    f, g = synth.make_case(kind, dims, seed, rel, decomp)
    return f.reshape(-1), g.reshape(-1)


def _bound(f, rel):
    return (f.max() - f.min()) * rel


def _mismatch(f, out, dims, want_saddles):
    L = O.cp_mismatch(O.pair(f, dims), O.pair(out, dims), dims)
    return [len(x) for x in L] if want_saddles else [len(L[0]), 0, 0, len(L[3])]


@pytest.mark.parametrize("dims,seed,rel", STALLING)
def test_reference_rules_stall(gpu_ctx, dims, seed, rel):
    """Without breaking, the loop runs into its round cap with mismatches left,
    as the oracle's does."""
    f, g = _case(dims, seed, rel)
    _, st, _ = O.correct(f, g, dims, rel, list(EXTREMA_ONLY), max_outer=5)
    assert not st["converged"]
    out = np.array(g, copy=True)
    rep = gpu_ctx.correct_ptr(f.ctypes.data, out.ctypes.data, dims, rel, EXTREMA_ONLY, on_device=False,
                              max_rounds=400, allow_nonconverged=True, break_stalls=False)
    assert not rep["converged"] and rep["stall_breaks"] == 0
    assert sum(rep["final_mismatch"]) > 0


@pytest.mark.parametrize("use_graph", [0, 1])
@pytest.mark.parametrize("dims,seed,rel", STALLING)
def test_breaking_converges(gpu_ctx, dims, seed, rel, use_graph):
    f, g = _case(dims, seed, rel)
    out, rep, cnt = gpu_ctx.correct(f, g, rel, EXTREMA_ONLY, dims=dims, max_rounds=20000, use_graph=use_graph,
                                    return_counter=True)
    assert rep["converged"] and rep["stall_breaks"] > 0
    assert sum(rep["final_mismatch"]) == 0
    # the oracle's loop with the same breaking rule, bit for bit
    want, st, wcnt = O.correct(f, g, dims, rel, list(EXTREMA_ONLY), max_outer=200, break_stalls=True)
    assert st["converged"] and st["oob"] == 0
    assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)
    assert rep["stall_breaks"] == st["stall_breaks"]
    assert rep["cp_rounds"] == st["cp_iterations"] and rep["outer_iterations"] == st["outer_iterations"]
    # and checked from scratch: within the bound, the original extrema, and
    # not everything back at the original
    assert np.all(np.abs(out - f) <= _bound(f, rel) * (1 + 1e-12))
    assert _mismatch(f, out, dims, False) == [0, 0, 0, 0]
    assert np.count_nonzero(out != f) > 0


@pytest.mark.parametrize("dims,seed,rel", STALLING[:2])
def test_breaking_same_in_both_loops(gpu_ctx, dims, seed, rel):
    f, g = _case(dims, seed, rel)
    a, ra = gpu_ctx.correct(f, g, rel, EXTREMA_ONLY, dims=dims, max_rounds=20000, use_graph=0)
    b, rb = gpu_ctx.correct(f, g, rel, EXTREMA_ONLY, dims=dims, max_rounds=20000, use_graph=1)
    assert np.array_equal(a, b)
    for k in ("stall_breaks", "cp_rounds", "path_rounds", "outer_iterations", "converged", "final_mismatch"):
        assert ra[k] == rb[k], k


@pytest.mark.parametrize("flags", [FULL, (1, 0, 0, 0, 0, 0, 0)])
@pytest.mark.parametrize("dims,kind,seed,rel,decomp", [((24, 20, 18), "powerlaw", 1, 1e-3, "sz"),
                                                       ((20, 18, 16), "gauss", 2, 1e-2, "uniform")])
def test_converging_runs_unchanged(gpu_ctx, dims, kind, seed, rel, decomp, flags):
    """Where the reference's rules converge, breaking never triggers and the
    output is the oracle's, bit for bit."""
    f, g = _case(dims, seed, rel, kind, decomp)
    want, st, wcnt = O.correct(f, g, dims, rel, list(flags), max_outer=500)
    if not st["converged"]:
        pytest.skip("the reference rules do not converge on this input")
    for use_graph in (0, 1):
        out, rep, cnt = gpu_ctx.correct(f, g, rel, flags, dims=dims, use_graph=use_graph, return_counter=True)
        assert rep["stall_breaks"] == 0
        assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)


def test_breaking_full_msc_in_batch(gpu_ctx):
    """The uneven batch's smallest fields under full-MSC flags: every field
    converges with breaking on; the ones that needed it stay within the bound
    and match the original's critical cells under the oracle."""
    from dmtz_gb300 import synth

    fields = [x for x in synth.batch_workload(64, lo=32, hi=64)][:16]
    res = gpu_ctx.correct_batch(fields, workers=4, max_rounds=20000)
    for (f, g, rel), (out, rep, st) in zip(fields, res):
        assert st == 0 and rep["converged"], rep
        ff = f.astype(np.float64)
        # every value the correction wrote is within the bound (float32 inputs
        # can be a rounding step outside it where nothing was written)
        wrote = out != g.astype(np.float64)
        assert np.all(np.abs(out - ff)[wrote] <= _bound(ff, rel) * (1 + 1e-12))
        if rep["stall_breaks"]:
            D, H, W = f.shape
            assert _mismatch(ff.reshape(-1), out.reshape(-1), (W, H, D), True) == [0, 0, 0, 0]


@pytest.mark.parametrize("use_graph", [0, 1])
def test_breaking_full_msc(gpu_ctx, use_graph):
    """A full-MSC case whose critical-point phase stalls under the reference's
    rules: breaking converges to the oracle's result, in which the oracle finds
    neither a critical-cell mismatch nor a separatrix record."""
    dims, seed, rel = (32, 28, 24), 1, 1e-2
    f, g = _case(dims, seed, rel)
    stuck = np.array(g, copy=True)
    rep0 = gpu_ctx.correct_ptr(f.ctypes.data, stuck.ctypes.data, dims, rel, FULL, on_device=False, max_rounds=600,
                               use_graph=use_graph, allow_nonconverged=True, break_stalls=False)
    assert not rep0["converged"]
    out, rep, cnt = gpu_ctx.correct(f, g, rel, FULL, dims=dims, max_rounds=20000, use_graph=use_graph,
                                    return_counter=True)
    assert rep["converged"] and rep["stall_breaks"] > 0
    want, st, wcnt = O.correct(f, g, dims, rel, list(FULL), max_outer=200, break_stalls=True)
    assert st["converged"]
    assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)
    assert rep["stall_breaks"] == st["stall_breaks"] and rep["outer_iterations"] == st["outer_iterations"]
    assert np.all(np.abs(out - f) <= _bound(f, rel) * (1 + 1e-12))
    P, Q = O.pair(f, dims), O.pair(out, dims)
    assert [len(x) for x in O.cp_mismatch(P, Q, dims)] == [0, 0, 0, 0]
    at, ac, de, dv, oob = O.path_detect(P, Q, dims)
    assert oob == 0 and len(at) == 0 and len(de) == 0
