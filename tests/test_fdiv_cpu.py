"""The multiply-high division of the cell id decodes, checked on the host
(nvcc compiles the header's host path; no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fdiv_exact(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "fdiv_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-o", exe, os.path.join(HERE, "native", "fdiv_check.cu")], check=True,
                   capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 wrong" in r.stdout
