"""The large-field generators' recipes, run on the CPU at small sizes."""
import numpy as np
import pytest


def test_gaussian_mix_device_recipe():
    torch = pytest.importorskip("torch")
    from dmtz_gb300 import synth

    dims, seed, n = (24, 20, 16), 3, 6
    f = synth.gaussian_mix_device(dims, seed, n_gauss=n, sigma=(1.5, 4.0), noise=1e-3, device="cpu").numpy()
    # the same draws, summed densely without the +-6 sigma boxes
    W, H, D = dims
    gen = torch.Generator(device="cpu")
    gen.manual_seed(seed)
    c = (torch.rand((n, 3), generator=gen, dtype=torch.float64) * torch.tensor([W, H, D], dtype=torch.float64)).numpy()
    s = (1.5 + 2.5 * torch.rand(n, generator=gen, dtype=torch.float64)).numpy()
    a = (2.0 * torch.rand(n, generator=gen, dtype=torch.float64) - 1.0).numpy()
    want = (torch.randn((D, H, W), generator=gen, dtype=torch.float64) * 1e-3).numpy()
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    for k in range(n):
        d2 = (x - c[k, 0]) ** 2 + (y - c[k, 1]) ** 2 + (z - c[k, 2]) ** 2
        want += a[k] * np.exp(-d2 / (2.0 * s[k] ** 2))
    assert f.dtype == np.float64 and f.shape == (W * H * D,)
    assert np.max(np.abs(f - want.reshape(-1))) < 1e-7
    assert np.ptp(f) > 0.1
