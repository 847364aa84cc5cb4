"""Shared test helpers.

Markers: `gpu` tests need a CUDA device and call the product through the C ABI
(libdmtz).  Everything else runs on the CPU: the oracle against the golden
fixtures, host logic, and the ABI surface of the built library.
"""
import glob
import hashlib
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdmtz")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def fixture_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


def load_fixture(path):
    """(meta, arrays, f, g) with the inputs regenerated from the fixture's parameters."""
    from oracle.ref_harness import case_fields

    z = np.load(path, allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    f, g = case_fields(meta["kind"], tuple(meta["dims"]), meta["seed"], meta["rel"], meta["decomp"], meta["kw"])
    f = f.reshape(-1)
    g = g.reshape(-1)
    return meta, z, f, g


def reference_fixed(z, g_base):
    """The reference's corrected field rebuilt from a fixture."""
    if "fixed_full" in z:
        return z["fixed_full"]
    out = np.array(g_base, copy=True)
    out[z["fixed_idx"]] = z["fixed_val"]
    return out


def reference_cnt(z, V):
    c = np.ones(V, np.int32)
    c[z["cnt_idx"]] = z["cnt_val"]
    return c


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import dmtz_gb300 as dm

    ctx = dm.Context(0)
    yield ctx
    ctx.close()
