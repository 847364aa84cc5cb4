"""Benchmark: time to full Morse-Smale-complex match on the 256^3 workload.

Workload (one per GPU, seed = rank): a 256^3 Gaussian random field with
power spectrum P(k) ~ k^-3 normalised to [0, 1] (float32 values widened to
float64), decompressed field = SZ-style pre-quantisation (bin 2 eps) + 5 % of
voxels with extra U[-eps, eps], clamped to f +- eps; eps = 1e-4 x range; the
reference's full-MSC flags (preserve saddles, separatrices, geometry).
A step is one complete correction: extract both complexes, iterate fix /
apply / re-extract until the complexes (critical cells and separatrices)
agree.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours       : libdmtz on the GPU.  value = voxels / device time per step
                    (inputs resident in HBM); e2e = the same through the public
                    API from pinned host buffers (H2D of f and g and D2H of the
                    corrected field inside the timed region).
--impl reference  : the reference's algorithm on the host cores: the C
                    restatement of main_3d.cu (the reference itself is CUDA
                    only and has no CPU path), all host threads, on a bounded
                    sample of the same workload (its first 96^3 corner block,
                    with the whole field's absolute bound).
Multi-GPU: independent fields per rank (replicas, weak scaling), barrier +
max over ranks of the timed region.  `--gpus N` without a launcher starts the
N ranks itself (torch.distributed.run on 127.0.0.1).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

SIZE = 256
REL_EPS = 1e-4
FLAGS = (1, 1, 1, 0, 0, 0, 0)
METRIC = "Mvox/s to full MSC match (256^3 power-law, eps=1e-4 x range, full-MSC flags)"
SAMPLE = 96  # CPU sample: first SAMPLE^3 corner block of the same fields (about 10-15 s of CPU work)


def workload(seed: int, size: int = SIZE):
    from dmtz_gb300 import synth

    f, g = synth.make_case("powerlaw", (size, size, size), seed, REL_EPS, "sz")
    return f.reshape(-1), g.reshape(-1)


def octant(a, size, n):
    return np.ascontiguousarray(a.reshape(size, size, size)[:n, :n, :n]).reshape(-1)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()  # the timed region starts once samples flow
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def bf16_peak():
    """Dense bf16 tensor peak (burst, for a kernel timed alone), TFLOP/s."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def sweep_traffic():
    """DRAM bytes per gradient sweep from the committed ncu summary, if present."""
    try:
        with open(os.path.join(REPO, "profiles", "sweep_traffic.json")) as fh:
            t = json.load(fh)
        return t
    except (OSError, ValueError):
        return None


def cpu_sample(f, g, threads: int):
    """The oracle (C restatement of the reference) on the first SAMPLE^3 corner
    block.  The block keeps the whole field's absolute bound (its relative eps
    is rescaled to its own value range), so g stays within the bound the
    correction enforces."""
    from oracle import oracle as O

    fs, gs = octant(f, SIZE, SAMPLE), octant(g, SIZE, SAMPLE)
    dims = (SAMPLE, SAMPLE, SAMPLE)
    rel = REL_EPS * float(f.max() - f.min()) / float(fs.max() - fs.min())
    t0 = time.perf_counter()
    out, st, _ = O.correct(fs, gs, dims, rel, list(FLAGS), max_outer=2000, threads=threads)
    dt = time.perf_counter() - t0
    return SAMPLE ** 3 / dt / 1e6, dt, st


def reference_cuda(f, g, ours_sha: str):
    """The reference's own CUDA program on the same field and GPU: main_3d.cu,
    built by oracle/ref_harness.py (one compile fix, the data prefix moved to
    a working directory) into oracle/_ref/dmtz_ref, run once with its file
    contract in a scratch directory.  Its time is its own additional_time
    (main_3d.cu:7155, the correction after the files are read) and its phase
    timers (:7187); its corrected field is compared with this build's.  A
    baseline only, like cpu_baseline: run once, on rank 0."""
    import hashlib
    import shutil
    import tempfile

    from oracle import ref_harness as R

    exe = os.path.join(R.REF_DIR, "dmtz_ref")
    if not os.path.exists(exe):
        return {"unavailable": "the reference program was not built on this host (oracle/_ref/dmtz_ref missing)"}
    wd = tempfile.mkdtemp(prefix="dmtz_refcuda_")
    name = f"bench{SIZE}"
    try:
        rel_s = R._prepare_workdir(wd, name, f, g, REL_EPS, "none")
        argv = [exe, f"{name},{SIZE},{SIZE},{SIZE}", repr(REL_EPS), "none"] + [str(x) for x in FLAGS]
        env = dict(os.environ, PATH=os.path.join(wd, "bin") + ":" + os.environ.get("PATH", ""))
        t0 = time.perf_counter()
        try:
            p = subprocess.run(argv, cwd=wd, env=env, capture_output=True, timeout=900)
            rc, out = p.returncode, p.stdout.decode(errors="replace")
        except subprocess.TimeoutExpired:
            return {"unavailable": "the reference program did not finish within 900 s"}
        wall = time.perf_counter() - t0
        rec = {"rc": rc, "wall_s": wall}
        fx = os.path.join(wd, f"mscz/fixed_decp_data/fixed_decp_{name}_{rel_s}.bin")
        if os.path.exists(fx):
            raw = open(fx, "rb").read()
            n = int(np.frombuffer(raw[:8], np.uint64)[0])
            fixed = np.frombuffer(raw[8:], np.float64)[:n]
            rec["output_bit_identical"] = hashlib.sha256(fixed.tobytes()).hexdigest() == ours_sha
        sdir = os.path.join(wd, "stat_result")
        for fn in sorted(os.listdir(sdir)):
            for line in open(os.path.join(sdir, fn)):
                if line.startswith("additional_time:") and "seconds" not in rec:
                    rec["seconds"] = float(line.split(":")[1])
                if line.startswith("iteration number:"):
                    rec["iteration_number"] = int(line.split(":")[1])
        for line in out.splitlines():
            if line.startswith("build_cells:"):
                rec["phase_timers_s"] = line.strip()
        if "seconds" in rec:
            rec["mvox_s"] = SIZE ** 3 / rec["seconds"] / 1e6
        return rec
    finally:
        shutil.rmtree(wd, ignore_errors=True)


def max_over_ranks(values, dist=None, device="cpu"):
    """Element-wise maximum of per-rank floats over the process group (the
    slowest rank sets the job time); the values themselves without one."""
    if dist is None:
        return [float(x) for x in values]
    import torch

    t = torch.tensor([float(x) for x in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def job_value(world: int, voxels_per_rank: int, seconds: float) -> float:
    """Whole-job Mvox/s: every rank corrects its own field of voxels_per_rank."""
    return world * voxels_per_rank / seconds / 1e6


def run_reference(args, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    f, g = workload(0)
    vals, times = [], []
    st = None
    for i in range(args.warmup + args.steps):
        v, dt, st = cpu_sample(f, g, threads)
        if i >= args.warmup:
            vals.append(v)
            times.append(dt)
    value = float(np.mean(vals))
    sample = (f"full correction of the first {SAMPLE}^3 corner block of the 256^3 workload fields, with the field's bound "
              f"({st['outer_iterations']} outer iterations), C restatement of main_3d.cu, {threads} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mvox/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"powerlaw {SIZE}^3 seed 0, sz decompression, eps=1e-4 x range, flags 1110000",
                       "sample": f"{SAMPLE}^3 corner block", "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": "Mvox/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mvox/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def learned_vs_plain(ctx, f_dev, g0_dev, g_dev, dims, args):
    """Train the proposal network on args.traces traces of 128^3 power-law
    fields (seeds 1000.., eps = 1e-4 x range, 10 epochs, deterministic), then
    time the plain loop and the learned warm start on the benchmark field
    (device seconds, median of 3 each) and report the rounds of each."""
    import torch

    import dmtz_gb300 as dm
    from dmtz_gb300 import learned

    t0 = time.perf_counter()
    traces, skipped = learned.make_traces(ctx, args.traces, (128, 128, 128), 1000, REL_EPS)
    gen_s = time.perf_counter() - t0
    net = dm.Network(0, seed=0)
    t1 = time.perf_counter()
    hist = learned.train(net, traces, epochs=10, lr=1e-3)
    train_s = time.perf_counter() - t1
    del traces
    torch.cuda.empty_cache()
    net.set_min_drop(args.min_drop[-1])
    res = {}
    for name in ("plain", "learned"):
        secs, rep = [], None
        for _ in range(3):
            g_dev.copy_(g0_dev)
            torch.cuda.synchronize()
            if name == "plain":
                rep = ctx.correct_ptr(f_dev.data_ptr(), g_dev.data_ptr(), dims, REL_EPS, FLAGS, on_device=True,
                                      use_graph=args.graph)
            else:
                rep = ctx.correct_learned_ptr(net, f_dev.data_ptr(), g_dev.data_ptr(), dims, REL_EPS, FLAGS,
                                              on_device=True, use_graph=args.graph)
            secs.append(rep["seconds"])
        res[name] = {"seconds": float(np.median(secs)), "cp_rounds": rep["cp_rounds"],
                     "path_rounds": rep["path_rounds"], "converged": rep["converged"],
                     "edited_vertices": rep["edited_vertices"]}
    net.close()
    k = max(1, len(hist) // 10)
    return {"plain": res["plain"], "learned": res["learned"],
            "speedup_plain_over_learned": res["plain"]["seconds"] / res["learned"]["seconds"],
            "training": {"traces": args.traces - len(skipped), "epochs": 10, "trace_generation_s": gen_s,
                         "train_s": train_s, "loss_first_epoch": float(np.mean(hist[:k])),
                         "loss_last_epoch": float(np.mean(hist[-k:])), "min_drop": args.min_drop[-1]},
            "note": "the network's edits are a warm start; the exact loop finishes, so values and labels stay exact"}


def run_ours(args, rank, world, local_rank):
    import torch

    import dmtz_gb300 as dm

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    dims = (SIZE, SIZE, SIZE)
    V = SIZE ** 3
    f, g = workload(rank)
    ctx = dm.Context(local_rank)
    f_dev = torch.from_numpy(f).cuda()
    g0_dev = torch.from_numpy(g).cuda()
    g_dev = g0_dev.clone()

    def step():
        g_dev.copy_(g0_dev)
        torch.cuda.synchronize()
        return ctx.correct_ptr(f_dev.data_ptr(), g_dev.data_ptr(), dims, REL_EPS, FLAGS, on_device=True,
                               use_graph=args.graph)

    rep = None
    for _ in range(args.warmup):
        rep = step()
    if not rep["converged"]:
        raise RuntimeError("correction did not converge")
    out = g_dev.cpu().numpy()
    bound = float(f.max() - f.min()) * REL_EPS
    ok_bound = bool(np.all(out - (f - bound) >= -1e-9 * bound))

    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    dev_s, launches = [], 0
    for _ in range(args.steps):
        r = step()
        dev_s.append(r["seconds"])
        launches += r["kernel_launches"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    clk = clocks.stop()
    t_step, wall = max_over_ranks([float(np.mean(dev_s)), wall], dist, "cuda")
    value = job_value(world, V, t_step)

    # end to end through the public API from pinned host buffers
    f_pin = torch.from_numpy(f).pin_memory()
    g0_pin = torch.from_numpy(g).pin_memory()
    g_pin = g0_pin.clone().pin_memory()
    g_pin.copy_(g0_pin)
    ctx.correct_ptr(f_pin.data_ptr(), g_pin.data_ptr(), dims, REL_EPS, FLAGS, on_device=False, use_graph=args.graph)
    e2e_t = []
    for _ in range(args.steps):
        g_pin.copy_(g0_pin)
        t1 = time.perf_counter()
        ctx.correct_ptr(f_pin.data_ptr(), g_pin.data_ptr(), dims, REL_EPS, FLAGS, on_device=False,
                        use_graph=args.graph)
        e2e_t.append(time.perf_counter() - t1)
    e2e_step = max_over_ranks([float(np.mean(e2e_t))], dist, "cuda")[0]

    # separatrix labels of the corrected field (g_dev holds the last timed
    # step's output): the reference's descending check looks at the first
    # vertex of each path only, so some descending labels may differ
    out_sha = None
    if rank == 0:
        import hashlib

        out_sha = hashlib.sha256(g_dev.cpu().numpy().tobytes()).hexdigest()
    agree = ctx.separatrix_agreement(f_dev.data_ptr(), g_dev.data_ptr(), dims, on_device=True)
    # the opt-in strict separatrix mode on the same field (not the reference's output)
    g_dev.copy_(g0_dev)
    torch.cuda.synchronize()
    srep = ctx.correct_ptr(f_dev.data_ptr(), g_dev.data_ptr(), dims, REL_EPS, FLAGS, on_device=True,
                           use_graph=args.graph, strict=True)
    sagree = ctx.separatrix_agreement(f_dev.data_ptr(), g_dev.data_ptr(), dims, on_device=True)

    # the reference arm's problem (the first SAMPLE^3 corner block, with the
    # whole field's bound) on the GPU, inputs resident in HBM
    fs, gs = octant(f, SIZE, SAMPLE), octant(g, SIZE, SAMPLE)
    rel_s = REL_EPS * float(f.max() - f.min()) / float(fs.max() - fs.min())
    fsd, gsd0 = torch.from_numpy(fs).cuda(), torch.from_numpy(gs).cuda()
    gsd = gsd0.clone()
    sdims = (SAMPLE, SAMPLE, SAMPLE)
    s_t = []
    for i in range(4):
        gsd.copy_(gsd0)
        torch.cuda.synchronize()
        r = ctx.correct_ptr(fsd.data_ptr(), gsd.data_ptr(), sdims, rel_s, FLAGS, on_device=True, use_graph=args.graph)
        if i:
            s_t.append(r["seconds"])

    # learned warm start against the plain loop on the same field (the
    # network trained here on 128^3 power-law traces; not timed above)
    learned_ab = None
    if rank == 0 and world == 1 and not args.no_learned:
        learned_ab = learned_vs_plain(ctx, f_dev, g0_dev, g_dev, dims, args)

    # roofline of the dominant kernel group: the gradient sweep run every round
    ms = ctx.profile_sweep(f_dev.data_ptr(), g0_dev.data_ptr(), dims, reps=20, on_device=True)
    alg_bytes = V * (2 * 8 + 1 / 8)  # read g and f, write a 1-bit mismatch flag per vertex
    achieved = alg_bytes / (ms[6] * 1e-3) / 1e9
    peak, peak_kind = peaks()
    tr = sweep_traffic()
    traffic = None
    if tr and tr.get("size") == SIZE:
        traffic = tr.get("bytes_per_sweep")

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mvox/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"powerlaw {SIZE}^3 seed=rank, sz decompression, eps=1e-4 x range, "
                                       f"flags {''.join(map(str, FLAGS))}",
                           "parallelism": f"replicas x{world}", "loop": "cuda graph" if args.graph else "host",
                           "l2": "inputs and state larger than L2 (f and g alone are 268 MB)",
                           "outer_iterations": rep["outer_iterations"], "cp_rounds": rep["cp_rounds"],
                           "path_rounds": rep["path_rounds"], "initial_mismatch": rep["initial_mismatch"],
                           "within_bound": ok_bound, "wall_s_per_step": wall / args.steps,
                           "phase_ms": rep["phase_ms"]},
                "time_to_match_s": t_step,
                "e2e": {"value": job_value(world, V, e2e_step), "unit": "Mvox/s", "seconds_per_step": e2e_step,
                        "h2d_bytes_per_step": 2 * V * 8, "d2h_bytes_per_step": V * 8 + 4},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                             "kernel": "gradient sweep (5 pairing passes + criticality)",
                             "sweep_ms": ms[6], "per_kernel_ms": [round(x, 4) for x in ms[:6]],
                             "step": {"definition": "the whole correction's least traffic: read f and g, "
                                                    "write the corrected g, 24 B/vertex, per step time",
                                      "achieved": 24.0 * V / t_step / 1e9,
                                      "frac": 24.0 * V / t_step / 1e9 / peak}},
                "clocks": clk, "gpu_launches": launches,
                "separatrix_agreement": {
                    "descending": agree["desc_equal"] / max(agree["desc_compared"], 1),
                    "ascending": agree["asc_equal"] / max(agree["asc_compared"], 1),
                    "critical_cells_differing": agree["crit_differ"], "counts": agree,
                    "note": "default (reference) loop: its descending check compares the first vertex of each path"},
                "strict_separatrices": {"seconds": srep["seconds"], "mvox_s": V / srep["seconds"] / 1e6,
                                        "outer_iterations": srep["outer_iterations"],
                                        "converged": srep["converged"],
                                        "descending": sagree["desc_equal"] / max(sagree["desc_compared"], 1),
                                        "ascending": sagree["asc_equal"] / max(sagree["asc_compared"], 1),
                                        "critical_cells_differing": sagree["crit_differ"]},
                "learned": learned_ab,
                "same_sample": {"workload": f"first {SAMPLE}^3 corner block, the field's bound (the reference arm's "
                                            f"problem)", "value": SAMPLE ** 3 / float(np.mean(s_t)) / 1e6,
                                "unit": "Mvox/s", "seconds": float(np.mean(s_t))}}
        if rank == 0 and world == 1 and not args.no_cpu:
            v, dt, st = cpu_sample(f, g, os.cpu_count() or 1)
            line["cpu_baseline"] = {"value": v, "unit": "Mvox/s", "cores": os.cpu_count() or 1, "kind": "port",
                                    "sample": f"oracle full correction of the first {SAMPLE}^3 corner block (field's bound), "
                                              f"{dt:.1f} s, {st['outer_iterations']} outer iterations"}
            if not args.no_ref_cuda:
                line["reference_cuda"] = reference_cuda(f, g, out_sha)
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_batch(args):
    """The uneven-batch workload: 64 fields (dims 32..192 per axis, float32 and
    float64, Gaussian-mix and power-law, eps in {1e-2,1e-3,1e-4} x range),
    corrected with dmtz_correct_batch; also timed with one worker (no overlap)."""
    import dmtz_gb300 as dm
    from dmtz_gb300 import synth

    t0 = time.perf_counter()
    fields = synth.batch_workload(64)
    gen_s = time.perf_counter() - t0
    vox = sum(f.size for f, _, _ in fields)
    ctx = dm.Context(0)
    f0, g0, _ = fields[0]
    shape, bps, _ = ctx.autotune(f0.astype(np.float64), g0.astype(np.float64))
    res = {}
    for workers in (8, 1):
        ctx.correct_batch(fields[:4], workers=workers, max_rounds=args.max_rounds)  # warm-up
        t1 = time.perf_counter()
        out = ctx.correct_batch(fields, workers=workers, max_rounds=args.max_rounds)
        dt = time.perf_counter() - t1
        res[workers] = (dt, sum(1 for o in out if o[1]["converged"]), sum(o[1]["stall_breaks"] for o in out),
                        sum(1 for o in out if o[1]["stall_breaks"]))
    line = {"metric": "Mvox/s, 64-field uneven batch corrected in one call (full-MSC flags)",
            "value": vox / res[8][0] / 1e6, "unit": "Mvox/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": res[8][0] * 1e3, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "64 fields, dims U{32..192}^3, f32/f64 alternating, gauss/powerlaw, "
                                   "eps in {1e-2,1e-3,1e-4} x range", "voxels": int(vox), "workers": 8,
                       "converged": res[8][1], "stall_breaks": res[8][2], "fields_with_stall_breaks": res[8][3],
                       "max_rounds": args.max_rounds, "tuning": [shape, bps],
                       "one_worker_s": res[1][0], "overlap_speedup": res[1][0] / res[8][0],
                       "generation_s": gen_s}}
    print(json.dumps(line), flush=True)
    ctx.close()


# tensor-core work of one forward pass per vertex, as executed: 3x3x3 taps,
# channels 16->32->32->32->16 (the last layer's 16 outputs are the MMA width;
# one is used)
CNN_FLOP_PER_VOX = 2 * 27 * (16 * 32 + 32 * 32 + 32 * 32 + 32 * 16)


def run_cnn(args):
    """Throughput of the learned-proposal network kernels on a SIZE^3 grid of
    the benchmark field's features: forward (inference), training step, and
    the dominant 32->32 convolution launch against the bf16 tensor peak."""
    import torch

    import dmtz_gb300 as dm

    size = args.cnn_size
    f, g = workload(0, size)
    dims = (size, size, size)
    V = size ** 3
    ctx = dm.Context(0)
    net = dm.Network(0, seed=0)
    net.set_tensor_path(args.tensor_path)
    fd, gd = torch.from_numpy(f).cuda(), torch.from_numpy(g).cuda()
    feat = torch.empty((V, 16), dtype=torch.bfloat16, device="cuda")
    active = torch.empty(V, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.features(fd.data_ptr(), gd.data_ptr(), dims, REL_EPS, feat.data_ptr(), active.data_ptr())
    out = torch.empty(V, dtype=torch.float32, device="cuda")
    target = torch.zeros(V, dtype=torch.float32, device="cuda")
    ones = torch.ones(V, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ms = net.profile(feat.data_ptr(), out.data_ptr(), target.data_ptr(), ones.data_ptr(), dims, reps=max(args.steps, 1))
    pk, pk_src = bf16_peak()
    conv_flop = 2 * 27 * 32 * 32 * V
    tf_conv = conv_flop / (ms[2] * 1e-3) / 1e12
    # the tensor pipe's own rate for the instruction shape the convolutions
    # use (128 x 32 x 16) and for wider ones, measured here
    ceil = {n: net.mma_ceiling(n) for n in (32, 64, 96, 128, 256)}
    # path 2's MMAs are 128 x 96 x 16, of whose 128 rows (16 per x-line) 14 are outputs
    shape_n, row_eff = (96, 14 / 16) if args.tensor_path == 2 else (32, 1.0)
    line = {"metric": "learned-proposal network, forward TFLOP/s (bf16 tensor cores)",
            "value": CNN_FLOP_PER_VOX * V / (ms[0] * 1e-3) / 1e12, "unit": "TFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": 1, "ms_per_step": ms[0], "higher_is_better": True, "dtype": "bf16",
            "data": "synthetic",
            "config": {"workload": f"features of the powerlaw {size}^3 benchmark field", "voxels": V,
                       "flop_per_voxel_forward": CNN_FLOP_PER_VOX, "train_step_ms": ms[1],
                       "train_step_tflops": 3 * CNN_FLOP_PER_VOX * V / (ms[1] * 1e-3) / 1e12,
                       "wgrad32_ms": ms[3], "wgrad32_tflops": conv_flop / (ms[3] * 1e-3) / 1e12},
            "roofline": {"bound": "tensor", "kernel": {0: "k_conv", 1: "k_conv_tc", 2: "k_conv_tcx"}[args.tensor_path]
                         + "<32,32> (one 32->32 layer)", "achieved": tf_conv,
                         "peak": pk, "unit": "TFLOP/s", "frac": tf_conv / pk, "peak_source": pk_src,
                         "traffic": None,
                         "mma_shape_tflops": {f"128x{n}x16": ceil[n] for n in ceil},
                         "mma_shape": f"128x{shape_n}x16", "output_rows_per_mma": row_eff,
                         "frac_of_shape": tf_conv / row_eff / ceil[shape_n]}}
    print(json.dumps(line), flush=True)
    net.close()
    ctx.close()


def run_learned(args):
    """Plain vs learned warm start: train the network on traces of 128^3
    power-law fields (seeds 1000.., eps=1e-4 x range, full-MSC flags), then
    correct held-out fields both ways and compare device time and rounds."""
    import dmtz_gb300 as dm
    from dmtz_gb300 import learned

    ctx = dm.Context(0)
    t0 = time.perf_counter()
    traces, skipped = learned.make_traces(ctx, args.traces, (128, 128, 128), 1000, REL_EPS)
    gen_s = time.perf_counter() - t0
    net = dm.Network(0, seed=0)
    t1 = time.perf_counter()
    hist = learned.train(net, traces, epochs=args.epochs, lr=args.lr)
    train_s = time.perf_counter() - t1
    if args.save_params:
        net.save(args.save_params)
    n_used = len(traces)
    del traces
    evals = []
    for size, seed in ((256, 0), (args.eval_size, 7)):
        from dmtz_gb300 import synth

        f, g = synth.make_case("powerlaw", (size,) * 3, seed, REL_EPS, "sz")
        learned.evaluate(ctx, net, f[:64, :64, :64], g[:64, :64, :64], REL_EPS, max_rounds=50)  # warm-up
        keep = ("seconds", "wall_s", "cp_rounds", "path_rounds", "outer_iterations", "converged", "edited_vertices",
                "max_err_over_bound", "initial_mismatch")
        ev = {"field": f"powerlaw {size}^3 seed {seed}"}
        best = None
        for md in args.min_drop:
            net.set_min_drop(md)
            r = learned.evaluate(ctx, net, f, g, REL_EPS, max_rounds=args.max_rounds)
            ev["plain"] = {x: r["plain"][x] for x in keep}
            ev[f"learned_min_drop_{md}"] = {x: r["learned"][x] for x in keep}
            sp = r["plain"]["seconds"] / r["learned"]["seconds"]
            ev[f"learned_min_drop_{md}"]["speedup"] = sp
            if r["learned"]["converged"] and (best is None or sp > best[1]):
                best = (md, sp)
        ev["best"] = best
        evals.append(ev)
    last = evals[-1]
    line = {"metric": "time to full MSC match: plain loop vs learned warm start",
            "value": last["best"][1] if last["best"] else None,
            "unit": "x (plain s / learned s, best threshold)", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": last["plain"]["seconds"] * 1e3, "higher_is_better": True, "dtype": "bf16+f64",
            "data": "synthetic",
            "config": {"workload": f"train {args.traces} x 128^3 traces, {args.epochs} epochs, lr {args.lr}; "
                                   f"evaluate 256^3 and {args.eval_size}^3", "trace_generation_s": gen_s,
                       "traces_used": n_used, "skipped_nonconverged_seeds": skipped,
                       "train_s": train_s, "train_steps": len(hist),
                       "loss_first_epoch": float(np.mean(hist[:max(1, len(hist) // max(args.epochs, 1))])),
                       "loss_last_epoch": float(np.mean(hist[-max(1, len(hist) // max(args.epochs, 1)):]))},
            "evaluations": evals}
    print(json.dumps(line), flush=True)
    net.close()
    ctx.close()


def run_big(args):
    """The largest single-GPU cases, generated on the GPU: a power-law field of
    size^3 (default 1024^3, seed 11, f32 values widened to f64), or with
    --big-kind gauss a float64 Gaussian mixture of 4096 Gaussians with widths
    U[4, 32] (768^3, seed 12); SZ-style decompression at eps = 1e-4 x range,
    full-MSC flags.  The reference cannot run either (its int32 edge and
    triangle counts overflow).  Times the correction on the device (inputs
    resident in HBM) and reports the device memory the context held."""
    import torch

    import dmtz_gb300 as dm
    from dmtz_gb300 import synth

    n = args.big_size
    dims = (n, n, n)
    gauss = args.big_kind == "gauss"
    seed = 12 if gauss else 11
    t0 = time.perf_counter()
    f = synth.gaussian_mix_device(dims, seed) if gauss else synth.power_law_device(dims, seed)
    torch.cuda.empty_cache()  # the generator's temporaries go back to the device
    ctx = dm.Context(0)
    g0 = torch.empty_like(f)
    ctx.quantize_ptr(f.data_ptr(), g0.data_ptr(), dims, REL_EPS, 0.05, seed)  # SZ-style model on the GPU
    eps = REL_EPS * float(f.max() - f.min())
    gen_s = time.perf_counter() - t0
    free0, total = torch.cuda.mem_get_info()
    g = g0.clone()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    rep = ctx.correct_ptr(f.data_ptr(), g.data_ptr(), dims, REL_EPS, FLAGS, True, args.max_rounds, args.graph,
                          allow_nonconverged=True)
    wall = time.perf_counter() - t1
    free1, _ = torch.cuda.mem_get_info()
    within = bool(((g - f).abs() <= eps * (1 + 1e-12)).all().item())
    V = n ** 3
    kind = "f64 Gaussian-mix (4096 Gaussians)" if gauss else "power-law"
    line = {"metric": f"Mvox/s to full MSC match ({n}^3 {kind}, eps=1e-4 x range, full-MSC flags)",
            "value": V / rep["seconds"] / 1e6, "unit": "Mvox/s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": rep["seconds"] * 1e3, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{'gauss-mix 4096 x U[4,32]' if gauss else 'powerlaw'} {n}^3 seed {seed} "
                                   f"generated on the GPU, decompressed by the library's "
                                   f"quantiser (bin 2 eps, 5% noise), eps=1e-4 x range, "
                                   f"flags {''.join(map(str, FLAGS))}", "voxels": V, "generation_s": gen_s,
                       "wall_s": wall, "converged": rep["converged"], "within_bound": within,
                       "outer_iterations": rep["outer_iterations"], "cp_rounds": rep["cp_rounds"],
                       "path_rounds": rep["path_rounds"], "initial_mismatch": rep["initial_mismatch"],
                       "final_mismatch": rep["final_mismatch"], "stall_breaks": rep["stall_breaks"],
                       "phase_ms": rep["phase_ms"], "context_device_gb": (free0 - free1) / 1e9, "device_total_gb": total / 1e9,
                       "bytes_per_vertex": (free0 - free1) / V}}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_batch_field(args):
    """One field of the uneven batch (host-driven loop, so that every kernel
    is its own launch for profilers): device time, rounds and phase times."""
    import dmtz_gb300 as dm
    from dmtz_gb300 import synth

    f, g, rel = synth.batch_workload(64)[args.batch_field]
    D, H, W = f.shape
    ctx = dm.Context(0)
    out, rep = ctx.correct(f.astype(np.float64), g.astype(np.float64), rel, dims=(W, H, D), max_rounds=args.max_rounds,
                           use_graph=0)
    print(json.dumps({"workload": f"batch field {args.batch_field}: {W}x{H}x{D} {f.dtype}, eps {rel} x range",
                      **{k: rep[k] for k in ("seconds", "cp_rounds", "path_rounds", "stall_breaks", "kernel_launches",
                                             "phase_ms", "converged")}}), flush=True)
    ctx.close()


def sweep_only(size: int):
    """Gradient sweep kernels alone (for kernel profilers): 3 timed sweeps."""
    import torch

    import dmtz_gb300 as dm

    f, g = workload(0, size)
    ctx = dm.Context(0)
    fd, gd = torch.from_numpy(f).cuda(), torch.from_numpy(g).cuda()
    ms = ctx.profile_sweep(fd.data_ptr(), gd.data_ptr(), (size, size, size), reps=3, on_device=True)
    print(json.dumps({"size": size, "per_kernel_ms": [round(x, 4) for x in ms[:6]], "sweep_ms": ms[6]}))
    ctx.close()


def free_port() -> int:
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def spawn_ranks(n: int, argv) -> int:
    """`bench.py --gpus N` started without a launcher: start the N ranks
    (one process per GPU, torch.distributed.run on 127.0.0.1) with the same
    arguments and return their exit status.  Rank 0 prints the JSON line."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={free_port()}", os.path.abspath(__file__), *argv]
    return subprocess.run(cmd).returncode


def dist_check(args, rank, world):
    """Launcher check without GPUs (gloo): every rank joins the group, the
    max over ranks of a rank-dependent time is taken, rank 0 prints it."""
    import torch.distributed as dist

    dist.init_process_group("gloo")
    t = max_over_ranks([0.5 + rank], dist, "cpu")[0]
    dist.barrier()
    if rank == 0:
        print(json.dumps({"world": dist.get_world_size(), "max_t": t, "n_gpus": args.gpus}), flush=True)
    dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip the run of the reference's CUDA program")
    ap.add_argument("--graph", type=int, default=1, help="1: loop as a CUDA graph with a device-side flag")
    ap.add_argument("--sweep-only", type=int, default=0, metavar="SIZE",
                    help="profiling aid: only time the gradient sweep on a SIZE^3 field of the same kind")
    ap.add_argument("--workload", choices=["field256", "batch", "cnn", "learned", "big"], default="field256")
    ap.add_argument("--big-size", type=int, default=0, help="big workload: grid size (default 1024 power-law, "
                    "768 gauss)")
    ap.add_argument("--big-kind", choices=["powerlaw", "gauss"], default="powerlaw", help="big workload: field kind")
    ap.add_argument("--max-rounds", type=int, default=2000)
    ap.add_argument("--cnn-size", type=int, default=256, help="cnn workload: grid size")
    ap.add_argument("--tensor-path", type=int, default=2, choices=[0, 1, 2],
                    help="cnn workload: 1 tcgen05, 2 tcgen05 with folded x-taps, 0 mma.sync")
    ap.add_argument("--traces", type=int, default=200, help="learned workload and line: training traces")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned warm start's A/B in the default line")
    ap.add_argument("--epochs", type=int, default=10, help="learned workload: epochs")
    ap.add_argument("--lr", type=float, default=1e-3, help="learned workload: Adam learning rate")
    ap.add_argument("--eval-size", type=int, default=512, help="learned workload: held-out field size")
    ap.add_argument("--save-params", default="", help="learned workload: write the trained parameters (.npy)")
    ap.add_argument("--min-drop", type=float, nargs="+", default=[0.25, 0.5, 1.0],
                    help="learned workload: proposal thresholds (x bound) to evaluate")
    ap.add_argument("--batch-field", type=int, default=-1, metavar="I",
                    help="profiling aid: correct field I of the uneven batch alone (host-driven loop)")
    ap.add_argument("--dist-check", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args.gpus, sys.argv[1:]))
    if args.dist_check:
        dist_check(args, int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)))
        return
    if args.batch_field >= 0:
        run_batch_field(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "cnn":
        run_cnn(args)
        return
    if args.workload == "learned":
        run_learned(args)
        return
    if args.workload == "big":
        if args.big_size <= 0:
            args.big_size = 768 if args.big_kind == "gauss" else 1024
        run_big(args)
        return
    if args.sweep_only:
        sweep_only(args.sweep_only)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
