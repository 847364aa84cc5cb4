"""The 64^3 extrema-only workload (flags 0000000, seeds 0..9) through the C
ABI against the reference's own runs (tests/golden/ref_c0_rounds.json; see
test_oracle_c0.py).  The reference's loop never ends on these inputs, so the
pin is its state: both initial gradients, the first round's requests and
delta buffer, and the field after every one of the first 24 rounds, which
the CUDA path must reproduce bit for bit with stall breaking off (the
reference's rules alone).  With stall breaking on (the default) every seed
converges, and the result equals the oracle's loop with the same breaking
rule, within the bound and with the original extrema."""
import numpy as np
import pytest

from oracle import oracle as O
from test_oracle_c0 import RECS, c0_case, sha

pytestmark = pytest.mark.gpu
EXTREMA_ONLY = (0, 0, 0, 0, 0, 0, 0)


@pytest.mark.parametrize("rec", RECS, ids=lambda r: r["name"])
def test_c0_gradients_and_first_round(gpu_ctx, rec):
    f, g, dims = c0_case(rec)
    for arrs, keys in ((gpu_ctx.extract(f, dims), ("PV", "PE", "PF", "PT")),
                       (gpu_ctx.extract(g, dims), ("QV", "QE", "QF", "QT"))):
        for a, k in zip(arrs, keys):
            assert sha(a) == rec[k + "_sha256"], k
    buf = gpu_ctx.fix_round(f, g, np.ones(f.size, np.int32), rec["rel"], 0, 0, dims)
    rng = float(f.max() - f.min())
    idx = np.nonzero(buf != -2000.0 * rng)[0].astype(np.int32)
    assert sha(idx) == rec["rounds"][0]["req_idx_sha"] and sha(buf[idx]) == rec["rounds"][0]["req_buf_sha"]


@pytest.mark.parametrize("rec", RECS, ids=lambda r: r["name"])
def test_c0_rounds_match_reference(gpu_ctx, rec):
    f, g, dims = c0_case(rec)
    for r in range(1, 25):
        for use_graph in ((0, 1) if r in (1, 7, 24) else (0,)):
            out = np.array(g, copy=True)
            rep = gpu_ctx.correct_ptr(f.ctypes.data, out.ctypes.data, dims, rec["rel"], EXTREMA_ONLY, on_device=False,
                                      max_rounds=r, use_graph=use_graph, allow_nonconverged=True, break_stalls=False)
            assert not rep["converged"] and rep["cp_rounds"] == r
            assert sha(out) == rec["rounds"][r - 1]["field_sha"], (r, use_graph)


@pytest.mark.parametrize("rec", [RECS[0], RECS[3]], ids=lambda r: r["name"])
def test_c0_stall_breaking_converges(gpu_ctx, rec):
    f, g, dims = c0_case(rec)
    want, st, wcnt = O.correct(f, g, dims, rec["rel"], list(EXTREMA_ONLY), max_outer=50, break_stalls=True, threads=4)
    assert st["converged"] and st["stall_breaks"] > 0
    for use_graph in (0, 1):
        out, rep, cnt = gpu_ctx.correct(f, g, rec["rel"], EXTREMA_ONLY, dims=dims, use_graph=use_graph,
                                        return_counter=True, max_rounds=20000)
        assert rep["converged"] and rep["stall_breaks"] == st["stall_breaks"]
        assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)
        assert rep["cp_rounds"] == st["cp_iterations"]
    bound = (f.max() - f.min()) * rec["rel"]
    assert np.all(np.abs(out - f) <= bound * (1 + 1e-12))
    L = O.cp_mismatch(O.pair(f, dims, 4), O.pair(out, dims, 4), dims)
    assert len(L[0]) == 0 and len(L[3]) == 0
