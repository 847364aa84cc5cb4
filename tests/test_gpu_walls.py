"""Wall checks (preserve_connectors = 1) on the GPU against the oracle: the
records of the per-2-saddle searches (including searches too long for the
first, per-thread tier), and whole corrections bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(kind, dims, seed, rel):
    from dmtz_gb300 import synth

    f, g = synth.make_case(kind, dims, seed, rel, "sz" if kind == "powerlaw" else "uniform")
    return f.reshape(-1), g.reshape(-1)


# the 64^3 Gaussian mixture has walls of thousands of faces: its searches run
# through the larger tiers
DETECT = [("powerlaw", (20, 18, 16), 1, 1e-3), ("gauss", (20, 18, 16), 2, 1e-2), ("powerlaw", (33, 17, 9), 5, 3e-3),
          ("gauss", (64, 64, 64), 1, 1e-2), ("powerlaw", (64, 64, 64), 0, 1e-3)]


@pytest.mark.parametrize("kind,dims,seed,rel", DETECT)
def test_wall_detect_matches_oracle(gpu_ctx, kind, dims, seed, rel):
    f, g = _case(kind, dims, seed, rel)
    ws, we = gpu_ctx.wall_detect(f, g, dims)
    wws, wwe, pops, oob = O.wall_detect(O.pair(f, dims), O.pair(g, dims), dims)
    assert oob == 0
    assert np.array_equal(ws, wws) and np.array_equal(we, wwe)
    assert len(ws) > 0
    ws0, _ = gpu_ctx.wall_detect(f, f, dims)
    assert len(ws0) == 0


@pytest.mark.parametrize("use_graph", [0, 1])
@pytest.mark.parametrize("flags", [(1, 1, 1, 0, 1, 0, 0), (1, 1, 0, 0, 1, 0, 0), (1, 1, 1, 0, 1, 0, 1)])
@pytest.mark.parametrize("kind,dims,seed,rel", [("powerlaw", (20, 18, 16), 1, 1e-3), ("gauss", (20, 18, 16), 2, 1e-2)])
def test_wall_correction_matches_oracle(gpu_ctx, kind, dims, seed, rel, flags, use_graph):
    f, g = _case(kind, dims, seed, rel)
    want, st, wcnt = O.correct(f, g, dims, rel, list(flags), max_outer=400, break_stalls=True)
    if not st["converged"]:
        pytest.skip("the oracle does not converge within its cap here")
    out, rep, cnt = gpu_ctx.correct(f, g, rel, flags, dims=dims, max_rounds=50000, use_graph=use_graph,
                                    return_counter=True)
    assert rep["converged"] and rep["final_walls"] == 0
    assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)
    assert rep["outer_iterations"] == st["outer_iterations"] and rep["stall_breaks"] == st["stall_breaks"]
    P, Q = O.pair(f, dims), O.pair(out, dims)
    assert len(O.wall_detect(P, Q, dims)[0]) == 0


@pytest.mark.parametrize("flags", [(1, 1, 1, 0, 1, 0, 0), (1, 1, 0, 0, 1, 0, 0), (0, 0, 0, 0, 0, 0, 0)])
@pytest.mark.parametrize("case", range(6), ids=["tiny2", "tiny3", "noncubic", "flat", "ties", "thin"])
def test_edge_cases_with_walls_and_breaking(gpu_ctx, case, flags):
    """The parity edge cases (2^3 and 3^3 grids, non-cubic and thin grids, a
    constant field, many ties) with walls and stall breaking, against the
    oracle bit for bit; every run converges."""
    from test_gpu_parity import EDGE_CASES, _edge_field

    name, dims, kind, seed = EDGE_CASES[case]
    f = _edge_field(kind, dims, seed)
    rng = float(f.max() - f.min()) or 1.0
    r = np.random.Generator(np.random.PCG64(seed + 99))
    g = f + r.uniform(-0.05 * rng, 0.05 * rng, size=f.size)
    want, st, wcnt = O.correct(f, g, dims, 0.05, list(flags), max_outer=300, break_stalls=True)
    assert st["converged"] and st["oob"] == 0
    for use_graph in (0, 1):
        out, rep, cnt = gpu_ctx.correct(f, g, 0.05, flags, dims=dims, max_rounds=50000, use_graph=use_graph,
                                        return_counter=True)
        assert rep["converged"] and rep["stall_breaks"] == st["stall_breaks"]
        assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)
