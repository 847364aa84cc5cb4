"""The GPU decompression model against a numpy restatement of the same
arithmetic and counter-based random numbers (bit for bit), and its bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _unit(seed, v, k):
    with np.errstate(over="ignore"):
        h = _mix64(np.uint64(seed) + GOLD * (np.uint64(2) * v.astype(np.uint64) + np.uint64(k + 1)))
    return (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def _quantize_np(f, rel, frac, seed):
    fmin = f.min()
    eps = (f.max() - fmin) * rel
    w = 2.0 * eps
    q = fmin + w * np.rint((f - fmin) / w)
    v = np.arange(f.size)
    sel = _unit(seed, v, 0) < frac
    q = np.where(sel, q + eps * (2.0 * _unit(seed, v, 1) - 1.0), q)
    return np.minimum(np.maximum(q, f - eps), f + eps), eps


@pytest.mark.parametrize("dims,seed,rel,frac", [((40, 33, 21), 3, 1e-3, 0.05), ((17, 64, 9), 12345678901, 1e-4, 0.5),
                                                ((8, 8, 8), 0, 1e-2, 0.0)])
def test_quantize_matches_numpy(gpu_ctx, dims, seed, rel, frac):
    from dmtz_gb300 import synth

    f = synth.power_law(dims, seed % 1000).reshape(-1)
    g = gpu_ctx.quantize(f, rel, frac, seed, dims=dims)
    want, eps = _quantize_np(f, rel, frac, seed)
    assert np.array_equal(g, want)
    assert np.abs(g - f).max() <= eps * (1 + 1e-12)  # f -+ eps rounded, as the reference's fallback value
    # same seed, same field; another seed, another field
    assert np.array_equal(gpu_ctx.quantize(f, rel, frac, seed, dims=dims), g)
    if frac > 0:
        assert not np.array_equal(gpu_ctx.quantize(f, rel, frac, seed + 1, dims=dims), g)


def test_quantized_field_corrects(gpu_ctx):
    from dmtz_gb300 import synth

    dims = (48, 40, 36)
    f = synth.power_law(dims, 9).reshape(-1)
    g = gpu_ctx.quantize(f, 1e-3, 0.05, 9, dims=dims)
    out, rep = gpu_ctx.correct(f, g, 1e-3, dims=dims, use_graph=1)
    assert rep["converged"] and sum(rep["initial_mismatch"]) > 0
