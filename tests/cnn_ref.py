"""Float64 CPU reference of the learned-proposal network (test helper).

Restates, in numpy, what the GPU kernels compute: 3x3x3 zero-padded
convolutions 16 -> 32 -> 32 -> 32 -> 16 (output channel 0 used), ReLU between
layers, the weighted tanh-MSE loss and its parameter gradient.
The arithmetic is float64; `emulate=True` rounds to bfloat16 (round to nearest
even) exactly where the GPU stores bfloat16: weights, features, the three
activations and the three data gradients and the loss gradient.  With that
emulation the only difference left is the order of the fp32 accumulations
on the tensor cores.

Arrays are (D, H, W, C) channels-last; tap = (dz+1)*9 + (dy+1)*3 + (dx+1);
parameters flat, per layer weights [27][out][in] then bias [out].
"""
from __future__ import annotations

import numpy as np

LAYERS = ((16, 32), (32, 32), (32, 32), (32, 16))


def n_params() -> int:
    return sum(27 * i * o + o for i, o in LAYERS)


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32).astype(np.float64)


def bf16_bits(x):
    """bfloat16 bit patterns (uint16) of x, nearest even."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def split(params):
    """Flat parameters -> list of (weights [27, out, in], bias [out])."""
    out, o = [], 0
    for ci, co in LAYERS:
        w = np.asarray(params[o:o + 27 * co * ci], np.float64).reshape(27, co, ci)
        o += 27 * co * ci
        b = np.asarray(params[o:o + co], np.float64)
        o += co
        out.append((w, b))
    return out


def _taps():
    for tap in range(27):
        yield tap, tap % 3 - 1, (tap // 3) % 3 - 1, tap // 9 - 1


def conv(x, w, flip=False):
    """out[v][n] = sum_tap sum_c w[tap][n][c] x[v + off(tap)][c] (v - off if flip), zero outside."""
    D, H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((D, H, W, w.shape[1]))
    for tap, dx, dy, dz in _taps():
        if flip:
            dx, dy, dz = -dx, -dy, -dz
        sl = xp[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]
        out += sl @ w[tap].T
    return out


def wgrad(act, dz):
    """dW[tap][n][c] = sum_v dz[v][n] act[v + off(tap)][c]."""
    D, H, W, C = act.shape
    ap = np.pad(act, ((1, 1), (1, 1), (1, 1), (0, 0)))
    g = np.zeros((27, dz.shape[-1], C))
    dzf = dz.reshape(-1, dz.shape[-1])
    for tap, dx, dy, dzz in _taps():
        sl = ap[1 + dzz:1 + dzz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :].reshape(-1, C)
        g[tap] = dzf.T @ sl
    return g


def forward(feat, params, emulate=True):
    """feat (D, H, W, 16) -> (o (D, H, W), activations [a1, a2, a3])."""
    q = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    layers = split(params)
    x = q(feat)
    acts = []
    for l, (w, b) in enumerate(layers):
        z = conv(x, q(w)) + b
        if l < 3:
            x = q(np.maximum(z, 0.0))
            acts.append(x)
        else:
            o = z[..., 0]
    return o, acts


def loss_and_grad(feat, params, target, active, emulate=True):
    """Weighted mean sum w (tanh(o) - target)^2 / sum w (w = active, a 0/1 mask
    or byte weights) and its flat gradient."""
    q = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    layers = split(params)
    o, acts = forward(feat, params, emulate)
    y = np.tanh(o)
    w = np.asarray(active, np.float64)
    cnt = w.sum() if w.sum() > 0 else 1.0
    e = y - target
    loss = float((w * e ** 2).sum() / w.sum()) if w.sum() > 0 else 0.0
    dz4 = np.zeros(o.shape + (16,))
    dz4[..., 0] = 2.0 * w * e * (1.0 - y * y)
    dz = q(dz4)
    ins = [q(feat)] + acts
    grads = [None] * 4
    for l in range(3, -1, -1):
        w, _ = layers[l]
        gw = wgrad(ins[l], dz) / cnt
        gb = dz.reshape(-1, dz.shape[-1]).sum(0) / cnt
        grads[l] = (gw, gb)
        if l > 0:
            dprev = conv(dz, q(w).transpose(0, 2, 1), flip=True)
            dz = q(np.where(ins[l] > 0, dprev, 0.0))
    flat = np.concatenate([np.concatenate([gw.reshape(-1), gb]) for gw, gb in grads])
    return loss, flat
