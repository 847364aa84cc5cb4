"""The `dmtz` executable as a drop-in for the reference program: same argv,
same input files, and byte-identical output files (corrected field, edit
index file, edit value file) and stat lines, checked against what the
reference itself wrote for the same cases (tests/golden)."""
import json
import os
import stat
import subprocess

import numpy as np
import pytest

from conftest import REPO, fixture_files, load_fixture, reference_fixed

pytestmark = pytest.mark.gpu
EXE = os.path.join(REPO, "dmtz_gb300", "_lib", "dmtz")
CASES = [p for p in fixture_files() if "file_data_edits" in np.load(p).files]


def _layout(tmp, name, f, g, rel):
    root = os.path.join(tmp, "mscz")
    for d in ("decompressed_data", "compressed_data", "fixed_decp_data"):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    os.makedirs(os.path.join(tmp, "stat_result"), exist_ok=True)
    os.makedirs(os.path.join(tmp, "bin"), exist_ok=True)
    f.astype(np.float64).tofile(os.path.join(tmp, name + ".bin"))
    eps = "%.6e" % rel
    g.astype(np.float64).tofile(os.path.join(root, f"decompressed_data/decp_{name}_{eps}none_.bin"))
    with open(os.path.join(root, f"compressed_data/compressed_{name}_{eps}.sz"), "wb") as fh:
        fh.write(b"\0" * 4096)  # the same stand-in size the reference run used
    z = os.path.join(tmp, "bin", "zstd")
    with open(z, "w") as fh:
        fh.write('#!/bin/sh\nfor a in "$@"; do f="$a"; done\ncp "$f" "$f.zst"\n')
    os.chmod(z, os.stat(z).st_mode | stat.S_IEXEC)
    return root, eps


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[4:-4])
def test_cli_matches_reference_files(tmp_path, path):
    from dmtz_gb300 import build

    build.build()
    meta, z, f, g = load_fixture(path)
    W, H, D = meta["dims"]
    name = meta["name"]
    tmp = str(tmp_path)
    root, eps = _layout(tmp, name, f, g, meta["rel"])
    env = dict(os.environ, DMTZ_DATA_ROOT=root, PATH=os.path.join(tmp, "bin") + ":" + os.environ["PATH"])
    argv = [EXE, f"{name},{W},{H},{D}", repr(meta["rel"]), "none"] + [str(x) for x in meta["flags"]]
    p = subprocess.run(argv, cwd=tmp, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    raw = open(os.path.join(root, f"fixed_decp_data/fixed_decp_{name}_{eps}.bin"), "rb").read()
    assert int(np.frombuffer(raw[:8], np.uint64)[0]) == f.size
    assert np.array_equal(np.frombuffer(raw[8:], np.float64), reference_fixed(z, g))
    for key, stem in (("file_data1", "data1"), ("file_data", "data"), ("file_data_edits", "data_edits")):
        if key in z:
            got = open(os.path.join(root, f"{stem}{name}.bin"), "rb").read()
            assert got == z[key].tobytes(), stem
    # stat lines: everything but the two timings is determined by the outputs
    want = [ln for ln in meta["stat_result_text"].splitlines() if not ln.startswith(("compression_time", "additional_time"))]
    got = open(os.path.join(tmp, "stat_result", meta["stat_result_file"])).read().splitlines()
    got = [ln for ln in got if not ln.startswith(("compression_time", "additional_time"))]
    assert got == want
