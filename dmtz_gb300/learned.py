"""Learned proposal: training traces, the trainer, and the plain-vs-learned
comparison.  The network and every kernel run in libdmtz (dmtz_cnn_*,
dmtz_features, dmtz_correct_learned); this module only sequences the calls and
holds device buffers (torch tensors used as plain CUDA allocations).

A trace is what the exact correction did to one field:
    input   features of (f, g0) (16 bf16 channels per vertex) and the active
            mask (vertices within 2 of a criticality mismatch);
    target  (g_final - f) / bound in [-1, 1], g_final = the corrected field.
Training minimises mean (tanh(o) - target)^2 over active vertices with Adam.

At inference dmtz_correct_learned sets an active vertex to f + bound * tanh(o)
where that lowers g by at least min_drop x bound, then runs the exact loop, so
the output keeps
the loop's guarantees whatever the network predicts; the network can only
change how many rounds the loop needs.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import Context, Network, synth

FULL_MSC = (1, 1, 1, 0, 0, 0, 0)


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("the learned proposal needs a CUDA device")
    return torch


@dataclass
class Trace:
    dims: tuple
    feat: object      # torch bf16 (V, 16), device
    active: object    # torch uint8 (V,), device: loss weight, 0 outside the active mask
    target: object    # torch float32 (V,), device
    n_active: int
    report: dict = field(default_factory=dict)


def trace_fields(dims, seed, rel_eps, kind="powerlaw"):
    """(f, g0) of one training field: power-law (or Gaussian-mix) field and its
    SZ-style decompression (quantisation bin 2 eps plus 5% noise)."""
    f, g = synth.make_case(kind, dims, seed, rel_eps, "sz")
    return f, g


def make_trace(ctx: Context, f, g, rel_eps, flags=FULL_MSC, max_rounds=2000, use_graph=1, edit_weight=8):
    """Trace of one field, or None when the exact loop does not converge
    within max_rounds (the reference's loop can stall on such fields).  The
    loss weight of an active vertex is 1, or edit_weight where the loop
    changed its value (those are rare and are what the proposal must find)."""
    torch = _torch()
    f = np.ascontiguousarray(f, np.float64)
    D, H, W = f.shape
    dims = (W, H, D)
    V = W * H * D
    fd = torch.from_numpy(f.reshape(-1)).cuda()
    gd = torch.from_numpy(np.ascontiguousarray(g, np.float64).reshape(-1)).cuda()
    feat = torch.empty((V, 16), dtype=torch.bfloat16, device="cuda")
    active = torch.empty(V, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.features(fd.data_ptr(), gd.data_ptr(), dims, rel_eps, feat.data_ptr(), active.data_ptr())
    gfix = gd.clone()
    torch.cuda.synchronize()
    # traces follow the reference's rules only: a stalled field is skipped
    rep = ctx.correct_ptr(fd.data_ptr(), gfix.data_ptr(), dims, rel_eps, flags, True, max_rounds, use_graph,
                          allow_nonconverged=True, break_stalls=False)
    if not rep["converged"]:
        return None
    bound = rel_eps * float(f.max() - f.min())
    target = ((gfix - fd) / bound).clamp_(-1.0, 1.0).float() if bound > 0 else torch.zeros_like(gfix).float()
    n_active = int(active.sum().item())
    weight = active * torch.where(gfix != gd, int(edit_weight), 1).to(torch.uint8)
    return Trace(dims, feat, weight, target, n_active, rep)


def make_traces(ctx: Context, n, dims=(128, 128, 128), seed0=1000, rel_eps=1e-4, flags=FULL_MSC, log=None):
    """Traces of fields seed0, seed0+1, ...; fields whose exact loop does not
    converge are skipped.  Returns (traces, skipped seeds)."""
    out, skipped = [], []
    for i in range(n):
        f, g = trace_fields(dims, seed0 + i, rel_eps)
        tr = make_trace(ctx, f, g, rel_eps, flags)
        if tr is None:
            skipped.append(seed0 + i)
            continue
        out.append(tr)
        if log:
            log(f"trace {i}: active {tr.n_active}, rounds {tr.report.get('cp_rounds')}")
    return out, skipped


def train(net: Network, traces, epochs=10, lr=1e-3, seed=0, log=None):
    """Adam over the traces (one trace per step, shuffled each epoch).
    Returns the loss of every step."""
    torch = _torch()
    use = [t for t in traces if t.n_active > 0]
    if not use:
        return []
    vmax = max(int(np.prod(t.dims)) for t in use)
    out = torch.empty(vmax, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        for i in rng.permutation(len(use)):
            t = use[i]
            net.forward(t.feat.data_ptr(), out.data_ptr(), t.dims, train=True)
            hist.append(net.backward(t.target.data_ptr(), t.active.data_ptr(), t.dims))
            net.step(lr)
        if log:
            k = len(use)
            log(f"epoch {ep}: mean loss {np.mean(hist[-k:]):.5f}")
    return hist


def evaluate(ctx: Context, net: Network, f, g, rel_eps, flags=FULL_MSC, max_rounds=2000, use_graph=1):
    """Plain and learned correction of the same field, timed on the device.
    Returns {"plain": report, "learned": report} (reports of dmtz_correct /
    dmtz_correct_learned, plus wall seconds of each call)."""
    torch = _torch()
    f = np.ascontiguousarray(f, np.float64)
    D, H, W = f.shape
    dims = (W, H, D)
    fd = torch.from_numpy(f.reshape(-1)).cuda()
    g0 = torch.from_numpy(np.ascontiguousarray(g, np.float64).reshape(-1)).cuda()
    res = {}
    for name in ("plain", "learned"):
        gd = g0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if name == "plain":
            rep = ctx.correct_ptr(fd.data_ptr(), gd.data_ptr(), dims, rel_eps, flags, True, max_rounds, use_graph,
                                  allow_nonconverged=True)
        else:
            rep = ctx.correct_learned_ptr(net, fd.data_ptr(), gd.data_ptr(), dims, rel_eps, flags, True, max_rounds,
                                          use_graph, allow_nonconverged=True)
        rep["wall_s"] = time.perf_counter() - t0
        bound = rel_eps * float(f.max() - f.min())
        rep["max_err_over_bound"] = float((gd - fd).abs().max().item() / bound) if bound > 0 else 0.0
        res[name] = rep
    return res
