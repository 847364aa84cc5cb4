"""Batched correction and the autotuner: results must not depend on batching,
on the number of workers, or on the sweep configuration."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields():
    from dmtz_gb300 import synth

    out = []
    specs = [((16, 16, 16), "gauss", 1, 1e-2, np.float64), ((20, 18, 22), "powerlaw", 1, 1e-3, np.float32),
             ((24, 20, 18), "powerlaw", 7, 1e-3, np.float64), ((16, 12, 10), "gauss", 5, 2e-2, np.float32),
             ((33, 17, 21), "powerlaw", 9, 1e-3, np.float64), ((12, 30, 14), "gauss", 3, 1e-2, np.float32)]
    for dims, kind, seed, rel, dt in specs:
        kw = {"n_gauss": 8} if kind == "gauss" else {}
        f, g = synth.make_case(kind, dims, seed, rel, "uniform", **kw)
        out.append((f.astype(dt), g.astype(dt), rel))
    return out


def test_batch_equals_single(gpu_ctx):
    fields = _fields()
    res = gpu_ctx.correct_batch(fields, workers=3, max_rounds=5000)
    for (f, g, rel), (out, rep, st) in zip(fields, res):
        D, H, W = f.shape
        want, wrep = gpu_ctx.correct(f.astype(np.float64), g.astype(np.float64), rel, dims=(W, H, D), max_rounds=5000)
        assert st == 0 and rep["converged"]
        assert np.array_equal(out.reshape(-1), want)
        assert rep["outer_iterations"] == wrep["outer_iterations"]


def test_batch_float32_matches_oracle(gpu_ctx):
    """The batch path's float32 fields (widened to float64 on the way in)
    against the oracle directly, not only against dmtz_correct: values and
    round counts, bit for bit."""
    from oracle import oracle as O

    fields = _fields()
    f32 = [x for x in fields if x[0].dtype == np.float32]
    assert len(f32) >= 2
    res = gpu_ctx.correct_batch(f32, workers=2, max_rounds=5000)
    for (f, g, rel), (out, rep, st) in zip(f32, res):
        D, H, W = f.shape
        want, wst, _ = O.correct(f.astype(np.float64).reshape(-1), g.astype(np.float64).reshape(-1), (W, H, D), rel,
                                 [1, 1, 1, 0, 0, 0, 0], max_outer=500, break_stalls=True)
        assert st == 0 and rep["converged"] and wst["converged"] and wst["oob"] == 0
        assert np.array_equal(out.reshape(-1), want)
        assert rep["outer_iterations"] == wst["outer_iterations"] and rep["stall_breaks"] == wst["stall_breaks"]


def test_tuning_does_not_change_results(gpu_ctx):
    from dmtz_gb300 import synth

    dims = (40, 36, 30)
    f, g = synth.make_case("powerlaw", dims, 3, 1e-3, "sz")
    base, _ = gpu_ctx.correct(f, g, 1e-3, dims=dims)
    saved = gpu_ctx.get_tuning()
    try:
        for shape in range(3):
            for bps in (4, 32):
                gpu_ctx.set_tuning(shape, bps)
                out, _ = gpu_ctx.correct(f, g, 1e-3, dims=dims)
                assert np.array_equal(out, base), (shape, bps)
        shape, bps, ms = gpu_ctx.autotune(f, g, dims)
        assert 0 <= shape < 3 and bps in (8, 16, 32, 64) and ms > 0
        out, _ = gpu_ctx.correct(f, g, 1e-3, dims=dims)
        assert np.array_equal(out, base)
    finally:
        gpu_ctx.set_tuning(*saved)


def test_autotune_cache(gpu_ctx, tmp_path):
    from dmtz_gb300 import autotune, synth

    dims = (32, 32, 32)
    f, g = synth.make_case("powerlaw", dims, 4, 1e-3, "sz")
    saved = gpu_ctx.get_tuning()
    try:
        path = str(tmp_path / "tune.json")
        a = autotune.tune(gpu_ctx, f, g, path=path)
        b = autotune.tune(gpu_ctx, f, g, path=path)
        assert a[:2] == b[:2] and b[2] is None  # second call read the cache
    finally:
        gpu_ctx.set_tuning(*saved)
