"""Autotuner front end: a JSON cache of sweep configurations.

The library measures (`Context.autotune`): for each brick shape (8x4x4,
16x4x2, 32x2x2 anchors) and 8/16/32/64 blocks per SM it times a full gradient
sweep and keeps the fastest.  This module remembers the answer per
(GPU name, grid size class, dtype) in a JSON file, so later runs on the same
kind of input skip the measurement:

    from dmtz_gb300 import autotune
    autotune.tune(ctx, f, g)          # measures once, then reads the cache

The cache file is $DMTZ_TUNE_CACHE, default ~/.cache/dmtz_gb300/tune.json.
The choice changes only speed; results are identical for every choice.
"""
from __future__ import annotations

import json
import os

import numpy as np


def cache_path() -> str:
    return os.environ.get("DMTZ_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "dmtz_gb300", "tune.json"))


def size_class(dims) -> str:
    """Grid sizes rounded up to powers of two: nearby sizes share a choice."""
    return "x".join(str(1 << max(int(d) - 1, 1).bit_length()) for d in dims)


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def key(ctx, dims, dtype) -> str:
    return f"{ctx.device_name()}|{size_class(dims)}|{np.dtype(dtype).name}"


def tune(ctx, f, g, dims=None, dtype=np.float64, path=None, force=False):
    """Apply the cached choice for this input class, measuring it first if needed.
    Returns (shape, blocks_per_sm, ms or None when taken from the cache)."""
    f = np.asarray(f)
    if dims is None:
        D, H, W = f.shape
        dims = (W, H, D)
    path = path or cache_path()
    data = _load(path)
    k = key(ctx, dims, dtype)
    if not force and k in data:
        shape, bps = data[k]["shape"], data[k]["blocks_per_sm"]
        ctx.set_tuning(shape, bps)
        return shape, bps, None
    shape, bps, ms = ctx.autotune(f, g, dims)
    data[k] = {"shape": shape, "blocks_per_sm": bps, "sweep_ms": ms}
    _store(path, data)
    return shape, bps, ms
