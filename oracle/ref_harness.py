"""Build and run the reference program to pin the oracle (test infrastructure).

Three sub-commands:

``prepare`` (run where the reference sources are mounted): copies main_3d.cu
  from the reference tree into oracle/_ref/ (git-ignored) with a fixed set of
  textual edits and nothing else:
    1. the stray '/' after ``return 1;`` (main_3d.cu:7195) is removed, the only
       change needed for the file to compile;
    2. the hard-coded data prefix /pscratch/sd/y/yuxiaoli/MSCz becomes ./mscz
       (relative to the working directory of a run);
    3. read-only instrumentation: after the initial pairings it writes the
       original and decompressed pairing arrays, and after every
       applyDeltaBuffer1 launch it writes the delta buffer and the field (for
       the first DMTZ_DUMP_ROUNDS rounds, default 400), and at the end the
       edit counters, to ./dumps/.  None of it changes what the program
       computes.  With DMTZ_STOP_AFTER_DUMPS set, the process exits after the
       last dumped round: for inputs on which the reference's loop never ends
       (its rules reach a fixed point with mismatches left), the dumped rounds
       are the output.
``build`` (on the GPU host): nvcc for sm_103a into oracle/_ref/dmtz_ref.
``run`` (on the GPU host): generates every pinned case with dmtz_gb300.synth,
  lays out the reference's file contract (input .bin, decompressed file, dummy
  compressed file, stat_result/, a stand-in ``zstd`` that copies), runs the
  binary under a time limit and packs the outputs into one .npz per case.
  tests/golden/make_fixtures.py turns those into the committed fixtures.

Only cases that the oracle shows to converge without out-of-range accesses are
listed, so the reference's host loop (which has no iteration cap) ends.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import shutil
import stat
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_DIR = os.path.join(HERE, "_ref")
# where the reference's main_3d.cu is read from (prepare) and where the runs
# lay out their working directories; both can be overridden
REF_SRC = os.environ.get("DMTZ_REFERENCE_SRC", "/root/reference/main_3d.cu")
RUN_ROOT = os.environ.get("DMTZ_REF_WORKDIR", os.path.join(tempfile.gettempdir(), "dmtz_ref_run"))

# name, field kind, dims (W,H,D), seed, rel_eps, decompression model, extra kwargs, flag sets
CASES = [
    ("g16", "gauss", (16, 16, 16), 1, 1e-2, "uniform", {"n_gauss": 8},
     [[1, 0, 0, 0, 0, 0, 0], [1, 1, 1, 0, 0, 0, 0], [1, 1, 1, 0, 0, 0, 1], [1, 0, 0, 1, 0, 0, 0],
      [1, 0, 0, 0, 0, 1, 0], [1, 1, 1, 0, 0, 1, 1]]),
    ("p201822", "powerlaw", (20, 18, 22), 1, 1e-3, "sz", {}, [[1, 1, 1, 0, 0, 0, 0], [1, 0, 0, 0, 0, 0, 1]]),
    ("t161210", "tiegauss", (16, 12, 10), 5, 2e-2, "uniform", {"n_gauss": 6}, [[1, 1, 1, 0, 0, 0, 0]]),
    ("g32", "gauss", (32, 32, 32), 5, 1e-3, "uniform", {"n_gauss": 16}, [[1, 1, 1, 0, 0, 0, 0]]),
    ("g32s3", "gauss", (32, 32, 32), 3, 1e-3, "uniform", {"n_gauss": 16}, [[1, 1, 1, 0, 0, 0, 0]]),
    ("p48", "powerlaw", (48, 48, 48), 3, 1e-4, "sz", {}, [[1, 1, 1, 0, 0, 0, 0]]),
    ("p64", "powerlaw", (64, 64, 64), 0, 1e-4, "sz", {}, [[1, 1, 1, 0, 0, 0, 0]]),
    ("g64", "gauss", (64, 64, 64), 0, 1e-3, "uniform", {}, [[1, 0, 0, 0, 0, 0, 0]]),
]
# The 64^3 extrema-only workload (sum of 32 Gaussians + N(0, 1e-3) noise,
# eps = 1e-3 x range, g = f + U[-eps, eps], flags 0000000) for seeds 0..9.
# The reference's loop never ends on any of them (its rules reach a fixed
# point with false maxima left), so these runs dump the initial pairings and
# the first STALL_ROUNDS rounds and stop; only digests are kept.
C0_CASES = [(f"g64s{s}", "gauss", (64, 64, 64), s, 1e-3, "uniform", {}, [[0, 0, 0, 0, 0, 0, 0]]) for s in range(10)]
STALL_ROUNDS = 24
# large cases: no dumps, only the corrected field's digest, iteration count and timings
BIG_CASES = [
    ("p256", "powerlaw", (256, 256, 256), 0, 1e-4, "sz", {}, [[1, 1, 1, 0, 0, 0, 0]]),
]


def flag_tag(flags):
    return "".join(str(int(x)) for x in flags)


def case_fields(kind, dims, seed, rel, decomp, kw):
    sys.path.insert(0, REPO)
    from dmtz_gb300 import synth

    if kind == "tiegauss":
        # heavy ties: values on a coarse grid, so the index tie-break decides
        f = synth.gaussian_mix(dims, seed, **kw)
        f = np.round(f * 16.0) / 16.0
        eps = rel * synth.value_range(f)
        g = np.round(synth.decompress_uniform(f, eps, seed) * 64.0) / 64.0
        g = np.clip(g, f - eps, f + eps)
        return f, g
    return synth.make_case(kind, dims, seed, rel, decomp, **kw)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# ----------------------------------------------------------------------------- prepare
DUMP_HELPER = r'''
// ---- harness instrumentation (read-only dumps) ----
static int dmtz_dump_on() { static int on = -1; if (on < 0) on = getenv("DMTZ_DUMP") != nullptr; return on; }
static void dmtz_dump(const char* tag, int idx, const void* dptr, size_t bytes) {
    if (!dmtz_dump_on()) return;
    std::vector<char> h(bytes);
    cudaMemcpy(h.data(), dptr, bytes, cudaMemcpyDeviceToHost);
    char name[256];
    snprintf(name, sizeof(name), "dumps/%s_%d.bin", tag, idx);
    FILE* fp = fopen(name, "wb");
    if (fp) { fwrite(h.data(), 1, bytes, fp); fclose(fp); }
}
static int dmtz_round = 0;
static int dmtz_round_cap() {
    static int cap = -1;
    if (cap < 0) { const char* e = getenv("DMTZ_DUMP_ROUNDS"); cap = e ? atoi(e) : 400; }
    return cap;
}
#define DMTZ_DUMP_ROUND() do { if (dmtz_round < dmtz_round_cap()) { \
    dmtz_dump("buf", dmtz_round, buffer_temp, size2 * sizeof(double)); \
    dmtz_dump("decp", dmtz_round, decp_temp, size2 * sizeof(double)); } dmtz_round++; \
    if (getenv("DMTZ_STOP_AFTER_DUMPS") && dmtz_round >= dmtz_round_cap()) exit(0); } while (0)
'''

DUMP_INITIAL = r'''
    dmtz_dump("PV", 0, vertices_temp, numVertices * sizeof(int));
    dmtz_dump("PE", 0, edges_temp, numEdges * sizeof(int));
    dmtz_dump("PF", 0, faces_temp, numFaces * sizeof(int));
    dmtz_dump("PT", 0, tetra_temp, numTetrahedras * sizeof(int));
    dmtz_dump("QV", 0, dec_vertices_temp, numVertices * sizeof(int));
    dmtz_dump("QE", 0, dec_edges_temp, numEdges * sizeof(int));
    dmtz_dump("QF", 0, dec_faces_temp, numFaces * sizeof(int));
    dmtz_dump("QT", 0, dec_tetra_temp, numTetrahedras * sizeof(int));
    dmtz_dump("decp0", 0, decp_temp, size2 * sizeof(double));
'''


def prepare(src=REF_SRC):
    text = open(src).read()
    edits = [
        ("return 1; /\n", "return 1;\n", 1),
        ("/pscratch/sd/y/yuxiaoli/MSCz", "./mscz", None),
        ("namespace fs = std::filesystem;\n", "namespace fs = std::filesystem;\n" + DUMP_HELPER, 1),
        ('\n    cout<<"simplification_end"<<endl;\n', '\n    cout<<"simplification_end"<<endl;\n' + DUMP_INITIAL, 1),
        ("applyDeltaBuffer1<<<gridSize, blockSize>>>(width, height, depth);",
         "applyDeltaBuffer1<<<gridSize, blockSize>>>(width, height, depth); cudaDeviceSynchronize(); DMTZ_DUMP_ROUND();",
         2),
        ("cudaMemcpy(delta_counter1.data(), counter_device, size2 * sizeof(int), cudaMemcpyDeviceToHost);",
         "cudaMemcpy(delta_counter1.data(), counter_device, size2 * sizeof(int), cudaMemcpyDeviceToHost); "
         "if (dmtz_dump_on()) { FILE* fp = fopen(\"dumps/cnt_0.bin\", \"wb\"); if (fp) { fwrite(delta_counter1.data(), sizeof(int), size2, fp); fclose(fp); } }",
         1),
    ]
    for old, new, n in edits:
        k = text.count(old)
        if n is not None and k != n:
            raise SystemExit(f"anchor {old[:40]!r} found {k} times, expected {n}")
        text = text.replace(old, new)
    os.makedirs(REF_DIR, exist_ok=True)
    out = os.path.join(REF_DIR, "main_3d_ref.cu")
    with open(out, "w") as fh:
        fh.write(text)
    print("wrote", out)


# ----------------------------------------------------------------------------- build
def build():
    exe = os.path.join(REF_DIR, "dmtz_ref")
    cmd = ["nvcc", "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fopenmp",
           "-w", os.path.join(REF_DIR, "main_3d_ref.cu"), "-o", exe]
    t = time.time()
    subprocess.run(cmd, check=True)
    print(f"built {exe} in {time.time() - t:.1f}s")
    return exe


# ----------------------------------------------------------------------------- run
def _prepare_workdir(wd, name, f, g, rel, cid):
    os.makedirs(wd, exist_ok=True)
    for d in ("mscz/decompressed_data", "mscz/compressed_data", "mscz/fixed_decp_data", "stat_result", "dumps", "bin"):
        os.makedirs(os.path.join(wd, d), exist_ok=True)
    f.astype(np.float64).tofile(os.path.join(wd, name + ".bin"))
    rel_s = "%.6e" % rel
    g.astype(np.float64).tofile(os.path.join(wd, f"mscz/decompressed_data/decp_{name}_{rel_s}{cid}_.bin"))
    with open(os.path.join(wd, f"mscz/compressed_data/compressed_{name}_{rel_s}.sz"), "wb") as fh:
        fh.write(b"\0" * 4096)
    z = os.path.join(wd, "bin", "zstd")
    with open(z, "w") as fh:
        fh.write('#!/bin/sh\n# stand-in for zstd: "zstd -f FILE" -> FILE.zst (a copy)\nfor a in "$@"; do f="$a"; done\ncp "$f" "$f.zst"\n')
    os.chmod(z, os.stat(z).st_mode | stat.S_IEXEC)
    return rel_s


def run(out_dir, only=None, timeout=240, big=False):
    exe = os.path.join(REF_DIR, "dmtz_ref")
    os.makedirs(out_dir, exist_ok=True)
    summary = []
    for name, kind, dims, seed, rel, decomp, kw, flagsets in (BIG_CASES if big else CASES):
        if only and name not in only:
            continue
        f, g = case_fields(kind, dims, seed, rel, decomp, kw)
        for flags in flagsets:
            tag = f"{name}_{flag_tag(flags)}"
            wd = os.path.join(RUN_ROOT, tag)
            shutil.rmtree(wd, ignore_errors=True)
            cid = "none"
            rel_s = _prepare_workdir(wd, name, f, g, rel, cid)
            W, H, D = dims
            argv = [exe, f"{name},{W},{H},{D}", repr(rel), cid] + [str(x) for x in flags]
            env = dict(os.environ, PATH=os.path.join(wd, "bin") + ":" + os.environ.get("PATH", ""))
            if not big:
                env["DMTZ_DUMP"] = "1"
            t = time.time()
            try:
                p = subprocess.run(argv, cwd=wd, env=env, capture_output=True, timeout=timeout)
                rc, so = p.returncode, p.stdout
            except subprocess.TimeoutExpired as e:
                rc, so = -999, (e.stdout or b"")
            wall = time.time() - t
            rec = {"tag": tag, "rc": rc, "wall_s": wall}
            res = {}
            fx = os.path.join(wd, f"mscz/fixed_decp_data/fixed_decp_{name}_{rel_s}.bin")
            if os.path.exists(fx):
                raw = open(fx, "rb").read()
                n = int(np.frombuffer(raw[:8], np.uint64)[0])
                res["fixed"] = np.frombuffer(raw[8:], np.float64)[:n].copy()
            dd = os.path.join(wd, "dumps")
            small = f.size <= 20000
            for k in ("PV", "PE", "PF", "PT", "QV", "QE", "QF", "QT"):
                p_ = os.path.join(dd, f"{k}_0.bin")
                if os.path.exists(p_):
                    arr = np.fromfile(p_, np.int32)
                    rec[k + "_sha256"] = sha(arr)
                    rec[k + "_ncrit"] = int((arr == -1).sum())
                    if small:
                        res[k] = arr
            if os.path.exists(os.path.join(dd, "cnt_0.bin")):
                res["cnt"] = np.fromfile(os.path.join(dd, "cnt_0.bin"), np.int32)
            if os.path.exists(os.path.join(dd, "decp0_0.bin")):
                res["decp0"] = np.fromfile(os.path.join(dd, "decp0_0.bin"), np.float64)
            # per apply round, the requested vertices (delta buffer != sentinel),
            # their buffer values and the field values after the apply
            rounds = 0
            r_round, r_idx, r_buf, r_val = [], [], [], []
            while os.path.exists(os.path.join(dd, f"buf_{rounds}.bin")):
                b = np.fromfile(os.path.join(dd, f"buf_{rounds}.bin"), np.float64)
                d = np.fromfile(os.path.join(dd, f"decp_{rounds}.bin"), np.float64)
                sentinel = -2000.0 * float(f.max() - f.min())
                idx = np.nonzero(b != sentinel)[0]
                r_round.append(np.full(idx.size, rounds, np.int32))
                r_idx.append(idx.astype(np.int32))
                r_buf.append(b[idx])
                r_val.append(d[idx])
                rounds += 1
            rec["rounds"] = rounds
            if rounds:
                res["req_round"] = np.concatenate(r_round)
                res["req_idx"] = np.concatenate(r_idx)
                res["req_buf"] = np.concatenate(r_buf)
                res["req_val"] = np.concatenate(r_val)
            # the side files of the reference's cost()/original_cost(): edit indices
            # (3-bit counter bitmap or delta-coded indices) and edit values
            for stem in ("data1", "data", "data_edits"):
                p_ = os.path.join(wd, "mscz", f"{stem}{name}.bin")
                if os.path.exists(p_):
                    res["file_" + stem] = np.frombuffer(open(p_, "rb").read(), np.uint8).copy()
            for fn in os.listdir(os.path.join(wd, "stat_result")):
                if fn.startswith("result_"):
                    rec["stat_result_file"] = fn
                    rec["stat_result_text"] = open(os.path.join(wd, "stat_result", fn)).read()
            perf = [x for x in os.listdir(os.path.join(wd, "stat_result")) if x.startswith("performance1")]
            if perf:
                txt = open(os.path.join(wd, "stat_result", perf[0])).read()
                rec["perf"] = txt
                for line in txt.splitlines():
                    if line.startswith("iteration number:"):
                        rec["iteration_number"] = int(line.split(":")[1])
            for fn in os.listdir(os.path.join(wd, "stat_result")):
                if fn.startswith("result_"):
                    for line in open(os.path.join(wd, "stat_result", fn)):
                        if line.startswith("additional_time:"):
                            rec["additional_time"] = float(line.split(":")[1])
            for line in so.decode(errors="replace").splitlines():
                if line.startswith("build_cells:"):
                    rec["phase_timers"] = line.strip()
            if big and "fixed" in res:
                rec["fixed_sha256"] = sha(res["fixed"])
                rec["changed"] = int((res["fixed"] != g.reshape(-1)).sum())
                res = {}
            rec["stdout_head"] = so[:4000].decode(errors="replace")
            rec["stdout_tail"] = so[-4000:].decode(errors="replace")
            fg = {} if big else {"f": f.reshape(-1), "g": g.reshape(-1)}
            np.savez_compressed(os.path.join(out_dir, tag + ".npz"), **fg,
                                meta=json.dumps({"name": name, "kind": kind, "dims": dims, "seed": seed, "rel": rel,
                                                 "decomp": decomp, "kw": kw, "flags": flags, **rec}), **res)
            summary.append({k: rec[k] for k in rec if k not in ("perf", "stdout_head", "stdout_tail")})
            print(json.dumps(summary[-1]), flush=True)
    with open(os.path.join(out_dir, "summary_big.json" if big else "summary.json"), "w") as fh:
        json.dump(summary, fh, indent=1)


def run_rounds(out_path, cases=C0_CASES, rounds=STALL_ROUNDS, timeout=120):
    """Digests of reference runs whose loop does not end: per case the inputs'
    and the eight initial pairing arrays' sha256, and per round r < rounds the
    requested vertices (delta buffer entries other than the sentinel), their
    buffer values and the whole field after the update, as sha256 and counts."""
    exe = os.path.join(REF_DIR, "dmtz_ref")
    out = []
    for name, kind, dims, seed, rel, decomp, kw, flagsets in cases:
        f, g = case_fields(kind, dims, seed, rel, decomp, kw)
        for flags in flagsets:
            tag = f"{name}_{flag_tag(flags)}"
            wd = os.path.join(RUN_ROOT, tag)
            shutil.rmtree(wd, ignore_errors=True)
            rel_s = _prepare_workdir(wd, name, f, g, rel, "none")
            W, H, D = dims
            argv = [exe, f"{name},{W},{H},{D}", repr(rel), "none"] + [str(x) for x in flags]
            env = dict(os.environ, PATH=os.path.join(wd, "bin") + ":" + os.environ.get("PATH", ""), DMTZ_DUMP="1",
                       DMTZ_DUMP_ROUNDS=str(rounds), DMTZ_STOP_AFTER_DUMPS="1")
            t = time.time()
            try:
                p = subprocess.run(argv, cwd=wd, env=env, capture_output=True, timeout=timeout)
                rc = p.returncode
            except subprocess.TimeoutExpired:
                rc = -999
            rec = {"name": name, "kind": kind, "dims": list(dims), "seed": seed, "rel": rel, "decomp": decomp,
                   "kw": kw, "flags": flags, "rc": rc, "wall_s": time.time() - t,
                   "f_sha": sha(f.reshape(-1)), "g_sha": sha(g.reshape(-1))}
            dd = os.path.join(wd, "dumps")
            for k in ("PV", "PE", "PF", "PT", "QV", "QE", "QF", "QT"):
                p_ = os.path.join(dd, f"{k}_0.bin")
                if os.path.exists(p_):
                    arr = np.fromfile(p_, np.int32)
                    rec[k + "_sha256"] = sha(arr)
                    rec[k + "_ncrit"] = int((arr == -1).sum())
            sentinel = -2000.0 * float(f.max() - f.min())
            per = []
            r = 0
            while os.path.exists(os.path.join(dd, f"buf_{r}.bin")):
                b = np.fromfile(os.path.join(dd, f"buf_{r}.bin"), np.float64)
                d = np.fromfile(os.path.join(dd, f"decp_{r}.bin"), np.float64)
                idx = np.nonzero(b != sentinel)[0].astype(np.int32)
                per.append({"n_req": int(idx.size), "req_idx_sha": sha(idx), "req_buf_sha": sha(b[idx]),
                            "field_sha": sha(d), "changed": int((d != g.reshape(-1)).sum())})
                r += 1
            rec["rounds"] = per
            shutil.rmtree(wd, ignore_errors=True)
            out.append(rec)
            print(json.dumps({k: rec[k] for k in ("name", "rc", "wall_s")} | {"rounds": len(per)}), flush=True)
    with open(out_path, "w") as fh:
        json.dump(out, fh, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["prepare", "build", "run", "rounds"])
    ap.add_argument("--src", default=REF_SRC, help="prepare: the reference's main_3d.cu")
    ap.add_argument("--out", default=os.path.join(REPO, "ref_runs"))
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--timeout", type=float, default=240)
    ap.add_argument("--big", action="store_true", help="run the large timing cases (no dumps)")
    a = ap.parse_args()
    if a.cmd == "prepare":
        prepare(a.src)
    elif a.cmd == "build":
        build()
    elif a.cmd == "rounds":
        run_rounds(os.path.join(a.out, "rounds_c0.json"))
    else:
        run(a.out, a.only, a.timeout, a.big)


if __name__ == "__main__":
    main()
