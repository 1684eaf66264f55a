"""The N > 1 path of bench.py on the CPU: independent replicas, one per rank,
with a gloo barrier and the slowest rank's time (no data-path collective).
World size 2 over 127.0.0.1; no GPU is touched."""
import io
import multiprocessing as mp
import os
import socket
import sys
from contextlib import redirect_stdout
from types import SimpleNamespace

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), LOCAL_RANK=str(rank),
                      WORLD_SIZE="2")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        r, lr, ws = bench.dist_env()
        # each replica timed its own K = 20 steps; rank 1 was the slower one
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
        rate = bench.whole_job_rate(20, ms / 1e3, ws)
        dist.barrier()
        q.put((r, lr, ws, ms, rate))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, (r, lr, ws, ms, rate) in enumerate(res):
        assert (r, lr, ws) == (rank, rank, 2)
        assert ms == 15.0  # the max over the ranks, the same on both
        assert rate == pytest.approx(2 * 20 / 0.015)  # all replicas' steps over the slowest time


def test_one_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(7.5, None) == 7.5
    assert bench.whole_job_rate(10, 0.5, 1) == 20.0


def test_reference_arm_runs_on_rank_0_only(monkeypatch):
    # under torchrun every rank but 0 exits at once, printing nothing
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with redirect_stdout(buf):
        rc = bench.run_reference(SimpleNamespace(steps=3, warmup=1, gpus=2))
    assert rc == 0 and buf.getvalue() == ""
