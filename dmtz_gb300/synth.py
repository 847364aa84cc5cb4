"""Seeded synthetic scalar fields and decompression-error models.

The reference ships no data and names no public dataset, so every workload is
generated here from a seed:

* ``gaussian_mix``: a sum of isotropic Gaussians with uniform centres, widths
  and amplitudes plus white noise (the 64^3 extrema-only workload).
* ``power_law``: a Gaussian random field with spectrum P(k) ~ k^-3, normalised
  to [0, 1] (the 256^3 full-MSC workload).
* ``decompress_uniform``: original + U[-eps, eps] (an error-bounded lossy
  compressor's error model).
* ``decompress_sz``: SZ-style pre-quantisation with bin 2*eps, 5 % of voxels
  with extra U[-eps, eps] noise, clamped to [f - eps, f + eps].

Arrays are shaped (D, H, W) in C order, so the flat index is x + y*W + z*W*H,
the vertex numbering of the reference.  Original fields are float32 values
widened to float64 (the reference reads float64 only); decompressed fields are
float64.
"""
from __future__ import annotations

import numpy as np


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def gaussian_mix(dims, seed: int, n_gauss: int = 32, sigma=(2.0, 8.0), noise: float = 1e-3) -> np.ndarray:
    """Sum of n_gauss isotropic Gaussians + N(0, noise) as float32 widened to float64."""
    W, H, D = dims
    r = _rng(seed)
    c = r.uniform(0.0, 1.0, size=(n_gauss, 3)) * np.array([W, H, D], np.float64)
    s = r.uniform(sigma[0], sigma[1], size=n_gauss)
    a = r.uniform(-1.0, 1.0, size=n_gauss)
    z, y, x = np.meshgrid(np.arange(D, dtype=np.float64), np.arange(H, dtype=np.float64),
                          np.arange(W, dtype=np.float64), indexing="ij")
    f = np.zeros((D, H, W), np.float64)
    for k in range(n_gauss):
        d2 = (x - c[k, 0]) ** 2 + (y - c[k, 1]) ** 2 + (z - c[k, 2]) ** 2
        f += a[k] * np.exp(-d2 / (2.0 * s[k] ** 2))
    f += r.normal(0.0, noise, size=f.shape)
    return f.astype(np.float32).astype(np.float64)


def power_law(dims, seed: int, slope: float = -3.0) -> np.ndarray:
    """Gaussian random field with P(k) ~ k^slope, min-max normalised to [0, 1]."""
    W, H, D = dims
    r = _rng(seed)
    white = r.standard_normal((D, H, W))
    spec = np.fft.rfftn(white)
    kz = np.fft.fftfreq(D)[:, None, None]
    ky = np.fft.fftfreq(H)[None, :, None]
    kx = np.fft.rfftfreq(W)[None, None, :]
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    amp = np.zeros_like(k)
    nz = k > 0
    amp[nz] = k[nz] ** (slope / 2.0)
    f = np.fft.irfftn(spec * amp, s=(D, H, W), axes=(0, 1, 2))
    f = (f - f.min()) / (f.max() - f.min())
    return f.astype(np.float32).astype(np.float64)


def value_range(f: np.ndarray) -> float:
    return float(f.max() - f.min())


def decompress_uniform(f: np.ndarray, eps: float, seed: int) -> np.ndarray:
    """g = f + U[-eps, eps] (float64)."""
    r = _rng(seed + 7919)
    return f + r.uniform(-eps, eps, size=f.shape)


def decompress_sz(f: np.ndarray, eps: float, seed: int, frac: float = 0.05) -> np.ndarray:
    """SZ-style pre-quantisation (bin 2 eps) + frac of voxels with U[-eps, eps], clamped to f +- eps."""
    r = _rng(seed + 104729)
    fmin = float(f.min())
    g = fmin + 2.0 * eps * np.round((f - fmin) / (2.0 * eps))
    sel = r.random(f.shape) < frac
    g = g + sel * r.uniform(-eps, eps, size=f.shape)
    return np.clip(g, f - eps, f + eps)


def make_case(kind: str, dims, seed: int, rel_eps: float, decomp: str = "uniform", **kw):
    """Return (f, g) float64 arrays of shape (D, H, W) for a named field kind."""
    if kind == "gauss":
        f = gaussian_mix(dims, seed, **kw)
    elif kind == "powerlaw":
        f = power_law(dims, seed, **kw)
    else:
        raise ValueError(kind)
    eps = rel_eps * value_range(f)
    if decomp == "uniform":
        g = decompress_uniform(f, eps, seed)
    elif decomp == "sz":
        g = decompress_sz(f, eps, seed)
    else:
        raise ValueError(decomp)
    return f, g


def batch_workload(n: int = 64, seed: int = 2024, lo: int = 32, hi: int = 192):
    """The uneven batch: n fields with dims drawn per axis from [lo, hi], even
    index float32 / odd float64, Gaussian mixture or power-law alternately, and
    eps per field from {1e-2, 1e-3, 1e-4} x range.  Returns a list of
    (f, g, rel_eps) with f, g of the field's dtype, shape (D, H, W)."""
    r = _rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(x) for x in r.integers(lo, hi + 1, size=3))
        rel = float(r.choice([1e-2, 1e-3, 1e-4]))
        kind = "gauss" if i % 4 in (0, 1) else "powerlaw"
        sub = int(r.integers(0, 2**31 - 1))
        if kind == "gauss":
            scale = float(np.mean(dims)) / 64.0
            f = gaussian_mix(dims, sub, n_gauss=32, sigma=(2.0 * scale, 8.0 * scale))
        else:
            f = power_law(dims, sub)
        eps = rel * value_range(f)
        g = decompress_uniform(f, eps, sub) if kind == "gauss" else decompress_sz(f, eps, sub)
        dt = np.float32 if i % 2 == 0 else np.float64
        out.append((f.astype(dt), g.astype(dt), rel))
    return out


def power_law_device(dims, seed: int, slope: float = -3.0):
    """Large power-law field generated on the GPU (torch is used only as a
    seeded random-number and FFT toolbox here, for fields too big to build in
    host memory quickly): the recipe of power_law with torch's CUDA generator
    instead of numpy's, so the values differ from the host recipe's for the
    same seed.  Returns f as a float64 device tensor of shape (D*H*W,) holding
    float32 values.  The decompressed field comes from the library's own
    quantiser (Context.quantize_ptr)."""
    import torch

    W, H, D = dims
    gen = torch.Generator(device="cuda")
    gen.manual_seed(int(seed))
    white = torch.randn((D, H, W), generator=gen, device="cuda", dtype=torch.float32)
    spec = torch.fft.rfftn(white)
    del white
    kz = torch.fft.fftfreq(D, device="cuda")[:, None, None]
    ky = torch.fft.fftfreq(H, device="cuda")[None, :, None]
    kx = torch.fft.rfftfreq(W, device="cuda")[None, None, :]
    k2 = kx * kx + ky * ky + kz * kz
    amp = torch.where(k2 > 0, k2.clamp_min(1e-30) ** (slope / 4.0), torch.zeros_like(k2))
    spec *= amp
    del amp, k2
    f = torch.fft.irfftn(spec, s=(D, H, W))
    del spec
    f = ((f - f.min()) / (f.max() - f.min())).reshape(-1).double()
    torch.cuda.synchronize()
    return f


def gaussian_mix_device(dims, seed: int, n_gauss: int = 4096, sigma=(4.0, 32.0), noise: float = 1e-3,
                        device: str = "cuda"):
    """Large Gaussian-mixture field generated on the GPU, kept in float64:
    n_gauss isotropic Gaussians with centres U[0, dims), widths U[sigma) and
    amplitudes U[-1, 1], plus N(0, noise).  A Gaussian is separable, so each is
    added as an outer product of three 1-D profiles over its box of +-6 sigma
    (the tail left out is below 2e-8 of its amplitude).  torch's CUDA generator
    draws the parameters and the noise.  Returns a float64 device tensor of
    shape (D*H*W,)."""
    import torch

    W, H, D = dims
    dev = device
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    c = torch.rand((n_gauss, 3), generator=gen, device=dev, dtype=torch.float64) * torch.tensor(
        [W, H, D], dtype=torch.float64, device=dev)
    s = sigma[0] + (sigma[1] - sigma[0]) * torch.rand(n_gauss, generator=gen, device=dev, dtype=torch.float64)
    a = 2.0 * torch.rand(n_gauss, generator=gen, device=dev, dtype=torch.float64) - 1.0
    f = torch.randn((D, H, W), generator=gen, device=dev, dtype=torch.float64) * noise
    cc, ss, aa = c.cpu().numpy(), s.cpu().numpy(), a.cpu().numpy()
    axes = [torch.arange(n, dtype=torch.float64, device=dev) for n in (W, H, D)]

    def profile(k, ax, n):
        lo = max(0, int(np.floor(cc[k, ax] - 6.0 * ss[k])))
        hi = min(n, int(np.ceil(cc[k, ax] + 6.0 * ss[k])) + 1)
        d = axes[ax][lo:hi] - float(cc[k, ax])
        return lo, hi, torch.exp(-(d * d) / (2.0 * float(ss[k]) ** 2))

    for k in range(n_gauss):
        x0, x1, gx = profile(k, 0, W)
        y0, y1, gy = profile(k, 1, H)
        z0, z1, gz = profile(k, 2, D)
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        f[z0:z1, y0:y1, x0:x1].add_((float(aa[k]) * gz)[:, None, None] * gy[None, :, None] * gx[None, None, :])
    if dev != "cpu":
        torch.cuda.synchronize()
    return f.reshape(-1)
