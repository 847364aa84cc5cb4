"""Build recipe for libdmtz (sm_103a) and the drop-in `dmtz` executable.

nvcc is called directly (no cmake, no torch extension machinery): two
translation units for the library (the correction path, dmtz.cu, and the
learned-proposal network, cnn.cu), compiled in parallel and linked into one
shared object, and one small host file for the executable, linked against it.
Outputs go to dmtz_gb300/_lib/ (git-ignored).
"""
from __future__ import annotations

import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libdmtz.so")
EXE = os.path.join(LIBDIR, "dmtz")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".inc", ".cpp", ".h"))] + [
        os.path.join(REPO, "include", "dmtz.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd))
    return r


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libdmtz.so and the dmtz executable if their sources changed."""
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _sources()
    jobs = []
    if force or _stale(LIB, deps):
        objs = []
        procs = []
        for tu in ("dmtz.cu", "cnn.cu"):
            obj = os.path.join(LIBDIR, tu.replace(".cu", ".o"))
            objs.append(obj)
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
                   *(["-Xptxas", "-v"] if verbose else []), "-o", obj, os.path.join(CSRC, tu)]
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
        for cmd, p in procs:
            out, err = p.communicate()
            if p.returncode != 0:
                sys.stderr.write(out + err)
                raise RuntimeError("build failed: " + " ".join(cmd))
            if verbose:
                sys.stdout.write(out + err)
        jobs.append([NVCC, *ARCH, "-shared", "-o", LIB, *objs])
    for job in jobs:
        r = _run(job)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
    # the executable is host code linked against the library beside it
    cli = os.path.join(CSRC, "dmtz_cli.cpp")
    if os.path.exists(cli) and (force or jobs or _stale(EXE, deps)):
        _run([NVCC, "-O3", "-std=c++17", "-o", EXE, cli, "-L" + LIBDIR, "-ldmtz", "-Xlinker", "-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
