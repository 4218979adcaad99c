"""The benchmark's multi-rank host logic on CPU (gloo, two ranks): the job
time is the slowest rank's, the job rate counts every rank's frames, only
rank 0 runs the reference arm, and every replica runs the same frames.
The loop itself does not shard (frame t + 1 needs frame t's pose and map),
so ranks exchange nothing but this one reduction."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench.dist_env() == (ws, rank, rank)
        slowest = bench.max_over_ranks(1.5 + rank)
        out.put((rank, slowest, bench.job_fps(ws, 280, slowest)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [2.5, 2.5]  # both ranks see the slower rank's time
    assert all(abs(g[2] - 2 * 280 / 2.5) < 1e-9 for g in got)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.job_fps(1, 280, 0.1) == pytest.approx(2800.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "make_frames", lambda *a, **k: called.append(a))
    args = argparse.Namespace(steps=3, warmup=3, gpus=2, config="c2")
    assert bench.run_reference(args) is None
    assert called == [] and capsys.readouterr().out == ""


def test_replicas_run_the_same_frames():
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    pytest.importorskip("synth")
    a, b = bench.make_frames(2, 0), bench.make_frames(2, 1)
    for fa, fb in zip(a, b):
        assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])
