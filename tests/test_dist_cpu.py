"""Multi-process logic of bench.py on the CPU (gloo, world size 2): the
replicas' max-over-ranks timing, the whole-job value, one field per rank,
and the reference arm printing on rank 0 only."""
import io
import os
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t, wall = bench.max_over_ranks([1.0 + rank, 10.0 - rank], dist, "cpu")
    f, g = bench.workload(rank, 16)
    dist.barrier()
    q.put((rank, t, wall, float(f.sum()), bench.job_value(world, 16 ** 3, t)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, t0, w0, s0, v0), (r1, t1, w1, s1, v1) = out
    assert t0 == t1 == 2.0 and w0 == w1 == 10.0  # the slowest rank sets the time
    assert s0 != s1  # each rank corrects its own field (seed = rank)
    assert v0 == v1 == 2 * 16 ** 3 / 2.0 / 1e6


def test_max_over_ranks_without_group():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks([3, 4.5]) == [3.0, 4.5]
    assert bench.job_value(1, 256 ** 3, 0.04) == pytest.approx(419.43, rel=1e-4)


def test_reference_arm_prints_on_rank0_only():
    sys.path.insert(0, REPO)
    import bench

    class A:
        steps, warmup, gpus = 1, 0, 2

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(A, 1)
    assert buf.getvalue() == ""


def test_reference_arm_line(monkeypatch):
    """The reference arm's JSON line carries the keys of the bench contract
    (a 24^3 sample here, to keep the CPU suite quick)."""
    sys.path.insert(0, REPO)
    import json

    import bench

    monkeypatch.setattr(bench, "SAMPLE", 24)

    class A:
        steps, warmup, gpus = 1, 0, 1

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(A, 0)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "dtype", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1


def test_gpus_flag_spawns_ranks():
    """`bench.py --gpus 2` without a launcher starts two ranks itself; they
    form one process group (gloo here) and rank 0 alone prints."""
    import json
    import subprocess

    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR",
                                                            "MASTER_PORT")}
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--dist-check"],
                       capture_output=True, text=True, timeout=300, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["world"] == 2 and lines[0]["max_t"] == 1.5 and lines[0]["n_gpus"] == 2
