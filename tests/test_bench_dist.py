"""Multi-rank bookkeeping of bench.py on CPU: two gloo ranks, as torchrun
would start them.  Each rank codes its own replica of the workload (weak
scaling, no data-path collective); the job's time is the slowest rank's,
and only rank 0 of the reference arm does any work."""
from __future__ import annotations

import io
import os
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.job_ms(100.0 * (rank + 1), world, "cpu")
        gbs = bench.job_gbs(10**9, 4, world, ms)
        # the reference arm: ranks other than 0 exit without work or output
        out = io.StringIO()
        if rank != 0:
            with redirect_stdout(out):
                bench.reference_arm(None)   # returns before reading its arguments
        q.put((rank, ms, gbs, out.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, gbs, out in res:
        assert ms == 200.0                       # max over ranks, seen by every rank
        assert gbs == pytest.approx(2 * 4 * 1e9 / 0.2 / 1e9)
        if rank:
            assert out == ""


def test_single_rank_is_local_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_ms(12.5, 1, "cpu") == 12.5
    assert bench.job_gbs(2 * 10**9, 5, 1, 1000.0) == pytest.approx(10.0)


def test_reference_arm_prints_the_bench_line():
    """`bench.py --impl reference` runs the reference's own CPU codec (its
    library compiled from its sources, else the oracle port) with no GPU and
    prints one JSON line of the bench contract, tagged as the reference."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--small", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["value"] > 0 and d["higher_is_better"] is True
    for key in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "scaling", "dtype", "data", "config"):
        assert key in d, key
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
