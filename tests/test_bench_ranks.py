"""The benchmark's multi-rank logic on CPU (gloo, world size 2): replicas
combine their timings by the maximum (the slowest replica ends the job), the
whole-job rate counts every replica's searches, and ranks other than 0 of the
reference arm return without work.  The search itself needs a GPU; this
covers what runs around it."""
import multiprocessing as mp
import os
import socket
import sys
import pathlib

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo")
    try:
        t = bench.reduce_max(1.5 + rank, "cpu")        # rank 1 is the slower one
        out.put((rank, t, bench.whole_job_rate(10, t, 2)))
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_rate_over_two_gloo_ranks():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]          # both see the maximum
    assert [r[2] for r in res] == [8.0, 8.0]          # 2 ranks x 10 searches / 2.5 s


def test_single_rank_passthrough(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "1")
    assert bench.reduce_max(3.25, "cpu") == 3.25
    assert bench.whole_job_rate(5, 2.0, 1) == 2.5


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(None) is None
    assert capsys.readouterr().out == ""
