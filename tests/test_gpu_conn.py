"""Connectivity-mode separatrices (flags preserve_vpath=1, preserve_geometry=0)
on the GPU against the oracle: the detection records, and whole corrections in
the host-driven and the graph loop, bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [((16, 14, 12), "powerlaw", 1, 1e-3), ((20, 18, 16), "powerlaw", 2, 1e-3), ((24, 20, 18), "powerlaw", 3, 1e-3),
         ((18, 16, 14), "gauss", 5, 1e-2), ((33, 17, 9), "powerlaw", 11, 3e-3), ((9, 31, 12), "gauss", 7, 2e-2)]


def _case(dims, kind, seed, rel):
    from dmtz_gb300 import synth

    kw = {"n_gauss": 8} if kind == "gauss" else {}
    f, g = synth.make_case(kind, dims, seed, rel, "sz" if kind == "powerlaw" else "uniform", **kw)
    return f.reshape(-1), g.reshape(-1)


@pytest.mark.parametrize("dims,kind,seed,rel", CASES)
def test_conn_detection_matches_oracle(gpu_ctx, dims, kind, seed, rel):
    f, g = _case(dims, kind, seed, rel)
    at, ac, de, dv = gpu_ctx.path_detect(f, g, dims, connectivity=True)
    wat, wac, wde, wdv, oob = O.path_detect(O.pair(f, dims), O.pair(g, dims), dims, connectivity=True)
    assert oob == 0
    assert sorted(zip(at.tolist(), ac.tolist())) == sorted(zip(wat.tolist(), wac.tolist()))
    assert sorted(zip(de.tolist(), dv.tolist())) == sorted(zip(wde.tolist(), wdv.tolist()))
    assert len(wat) + len(wde) > 0


@pytest.mark.parametrize("flags", [(1, 1, 0, 0, 0, 0, 0), (1, 1, 0, 1, 0, 0, 0), (1, 1, 0, 0, 0, 0, 1)])
@pytest.mark.parametrize("dims,kind,seed,rel", CASES[:4])
def test_conn_correction_matches_oracle(gpu_ctx, dims, kind, seed, rel, flags):
    f, g = _case(dims, kind, seed, rel)
    want, st, wcnt = O.correct(f, g, dims, rel, list(flags), max_outer=500)
    if not st["converged"]:
        pytest.skip("the reference rules do not converge on this input")
    for use_graph in (0, 1):
        out, rep, cnt = gpu_ctx.correct(f, g, rel, flags, dims=dims, max_rounds=20000, use_graph=use_graph,
                                        return_counter=True)
        assert np.array_equal(out, want), use_graph
        assert np.array_equal(cnt, wcnt)
        assert rep["outer_iterations"] == st["outer_iterations"]
        assert rep["converged"]
    # the result keeps every separatrix's ends
    P, Q = O.pair(f, dims), O.pair(want, dims)
    at, ac, de, dv, _ = O.path_detect(P, Q, dims, connectivity=True)
    assert len(at) == 0 and len(de) == 0


def test_conn_correction_256_keeps_ends(gpu_ctx):
    """The bench field in connectivity mode: converges, within the bound, and the
    GPU's own connectivity check finds nothing left."""
    from dmtz_gb300 import synth

    dims = (96, 96, 96)
    f, g = synth.make_case("powerlaw", dims, 0, 1e-4, "sz")
    f, g = f.reshape(-1), g.reshape(-1)
    out, rep = gpu_ctx.correct(f, g, 1e-4, (1, 1, 0, 0, 0, 0, 0), dims=dims, use_graph=1)
    assert rep["converged"] and sum(rep["final_mismatch"]) == 0
    assert np.abs(out - f).max() <= 1e-4 * (f.max() - f.min()) * (1 + 1e-12)
    at, ac, de, dv = gpu_ctx.path_detect(f, out, dims, connectivity=True)
    assert len(at) == 0 and len(de) == 0
