"""The C ABI surface: libdmtz builds for sm_103a and exports every entry point
that include/dmtz.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

from conftest import REPO


def _declared():
    text = open(os.path.join(REPO, "include", "dmtz.h")).read()
    return sorted(set(re.findall(r"\b(dmtz_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = _declared()
    for n in ("dmtz_ctx_create", "dmtz_extract", "dmtz_mismatch", "dmtz_fix_round", "dmtz_path_detect",
              "dmtz_correct"):
        assert n in names


def test_library_builds_and_exports_all_symbols():
    from dmtz_gb300 import build

    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_cell_counts_without_gpu():
    import numpy as np

    import dmtz_gb300 as dm
    from oracle import oracle as O

    for dims in ((2, 2, 2), (5, 6, 7), (64, 64, 64), (1024, 1024, 1024)):
        got = dm.cell_counts(dims)
        if dims[0] < 1024:
            assert got == O.counts(dims)
        V, E, F, T = got
        W, H, D = dims
        assert V == W * H * D and T == 6 * (W - 1) * (H - 1) * (D - 1)


def test_cli_builds_and_prints_usage():
    import subprocess

    from dmtz_gb300 import build

    build.build()
    p = subprocess.run([build.EXE], capture_output=True, text=True)
    assert p.returncode == 2 and "usage" in p.stderr


def test_autotune_size_class():
    from dmtz_gb300 import autotune

    assert autotune.size_class((256, 256, 256)) == "256x256x256"
    assert autotune.size_class((200, 33, 2)) == "256x64x2"
