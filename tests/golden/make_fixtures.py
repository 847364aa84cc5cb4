"""Turn reference runs into the committed golden fixtures.

Input: the .npz files that `python oracle/ref_harness.py run` writes on a GPU
host (one per case: the reference program main_3d.cu, built with its one
compile fix, run on seeded synthetic inputs).  Output: one small
tests/golden/ref_<case>.npz per case holding

  meta        json: generator parameters, flags, the reference's
              "iteration number", sha256 + critical-cell count of each of the
              eight pairing arrays (original / decompressed)
  f_sha, g_sha sha256 of the regenerated inputs (guards the generator)
  fixed_*     the corrected field: full array when small, otherwise the
              indices and values of the vertices the reference changed,
              plus a sha256 of the whole array
  cnt_*       indices/values of edit counters that are not 1
  r0_idx, r0_buf  first fix round: vertices whose delta buffer entry is not
              the sentinel, and the buffer values
  file_*      (small cases) the reference's edit-index and edit-value files
              (data1<name>.bin or data<name>.bin, data_edits<name>.bin)

Usage: python tests/golden/make_fixtures.py <directory of oracle/ref_harness.py run dumps>
"""
import glob
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def convert(src, dst_dir=HERE):
    z = np.load(src, allow_pickle=False)
    m = json.loads(str(z["meta"]))
    keep = {k: m[k] for k in ("name", "kind", "dims", "seed", "rel", "decomp", "kw", "flags", "iteration_number",
                              "rounds")}
    for k in ("PV", "PE", "PF", "PT", "QV", "QE", "QF", "QT"):
        keep[k + "_sha256"] = m[k + "_sha256"]
        keep[k + "_ncrit"] = m[k + "_ncrit"]
    f, g, fixed = z["f"], z["g"], z["fixed"]
    out = {"meta": json.dumps(keep), "f_sha": sha(f), "g_sha": sha(g), "fixed_sha": sha(fixed)}
    if f.size <= 20000:
        out["fixed_full"] = fixed
    base = z["decp0"] if "decp0" in z else g
    ch = np.nonzero(fixed != base)[0].astype(np.int32)
    out["fixed_idx"] = ch
    out["fixed_val"] = fixed[ch]
    cnt = z["cnt"]
    ci = np.nonzero(cnt != 1)[0].astype(np.int32)
    out["cnt_idx"] = ci
    out["cnt_val"] = cnt[ci].astype(np.int8)
    # side files of the reference's cost()/original_cost() (small cases only)
    if f.size <= 20000:
        for k in ("file_data1", "file_data", "file_data_edits"):
            if k in z:
                out[k] = z[k]
        if "stat_result_text" in m:
            keep["stat_result_file"] = m["stat_result_file"]
            keep["stat_result_text"] = m["stat_result_text"]
        out["meta"] = json.dumps(keep)
    if "req_round" in z:
        sel = z["req_round"] == 0
        out["r0_idx"] = z["req_idx"][sel].astype(np.int32)
        out["r0_buf"] = z["req_buf"][sel]
    name = f"ref_{m['name']}_{''.join(str(x) for x in m['flags'])}.npz"
    np.savez_compressed(os.path.join(dst_dir, name), **out)
    return name


if __name__ == "__main__":
    src_dir = sys.argv[1] if len(sys.argv) > 1 else "ref_runs"
    for fn in sorted(glob.glob(os.path.join(src_dir, "*.npz"))):
        print(convert(fn))
