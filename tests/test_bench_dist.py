"""bench.py's multi-rank logic on CPU: two gloo ranks on 127.0.0.1 — the
job time is the maximum over ranks, the job rate counts every rank's units,
and the reference arm runs on rank 0 only (other ranks exit 0 without work)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms = [120.0, 180.0][rank]
        job_ms = bench.max_over_ranks(ms, ws)
        rate = bench.job_rate(1000.0, ws, 4, job_ms)
        dist.barrier()
        q.put((rank, job_ms, rate))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in ps)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, job_ms, rate in got:
        assert job_ms == 180.0                       # the slowest rank's time on every rank
        assert rate == pytest.approx(2 * 1000.0 * 4 / 0.18)


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    called = []
    monkeypatch.setattr(bench, "oracle_system", lambda: called.append(1))
    assert bench.run_reference(type("A", (), {"cpu_steps": 1, "warmup": 0, "steps": 1})()) == 0
    assert not called
