"""Mismatch lists sized for what occurs: a context whose lists start with room
for one entry must grow them on demand and give the same results as a context
with the default reserve, in the host loop and in the graph loop (which stops,
grows the list and resumes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tiny_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import dmtz_gb300 as dm

    ctx = dm.Context(0)
    ctx.set_list_reserve(0.0, 1)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("flags", [(1, 1, 1, 0, 0, 0, 0), (1, 0, 0, 0, 0, 0, 0), (1, 1, 1, 1, 0, 0, 0)])
@pytest.mark.parametrize("use_graph", [0, 1])
def test_growing_lists_give_same_correction(gpu_ctx, tiny_ctx, flags, use_graph):
    from dmtz_gb300 import synth

    dims = (36, 30, 28)
    f, g = synth.make_case("powerlaw", dims, 4, 1e-3, "sz")
    want, wrep = gpu_ctx.correct(f, g, 1e-3, flags, dims=dims, max_rounds=3000, use_graph=use_graph)
    got, rep = tiny_ctx.correct(f, g, 1e-3, flags, dims=dims, max_rounds=3000, use_graph=use_graph)
    assert np.array_equal(got, want)
    for k in ("outer_iterations", "cp_rounds", "path_rounds", "initial_mismatch", "final_mismatch", "converged"):
        assert rep[k] == wrep[k], k
    assert sum(rep["initial_mismatch"]) > 4


def test_growing_lists_give_same_stage_outputs(gpu_ctx, tiny_ctx):
    from dmtz_gb300 import synth

    dims = (24, 20, 18)
    f, g = synth.make_case("powerlaw", dims, 2, 1e-3, "sz")
    a = gpu_ctx.mismatch(f, g, dims)
    b = tiny_ctx.mismatch(f, g, dims)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    pa = gpu_ctx.path_detect(f, g, dims)
    pb = tiny_ctx.path_detect(f, g, dims)
    assert all(np.array_equal(x, y) for x, y in zip(pa, pb))
    cnt = np.ones(f.size, np.int32)
    da = gpu_ctx.fix_round(f, g, cnt, 1e-3, 1, 0, dims)
    db = tiny_ctx.fix_round(f, g, cnt, 1e-3, 1, 0, dims)
    assert np.array_equal(da, db)


def test_list_reserve_rejects_bad_arguments(tiny_ctx):
    import dmtz_gb300 as dm

    with pytest.raises(dm.DmtzError):
        tiny_ctx.set_list_reserve(1.5, 1)
    with pytest.raises(dm.DmtzError):
        tiny_ctx.set_list_reserve(0.1, 0)
