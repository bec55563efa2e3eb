"""bench.py's multi-rank bookkeeping on CPU (gloo, world size 2): ranks are
replicas, the whole-job rate is the sum of the ranks' units over the slowest
rank's time, and the reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = [1000.0, 3000.0][rank]
        secs = [2.0, 4.0][rank]
        rate, t = bench.whole_job_rate(units, secs)
        q.put((rank, rate, t))
    finally:
        dist.destroy_process_group()


def test_whole_job_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for _, rate, t in got:
        assert t == 4.0                      # the slowest rank's time
        assert rate == pytest.approx(4000.0 / 4.0)  # all ranks' units over it


def test_whole_job_rate_single_process():
    assert bench.whole_job_rate(10.0, 4.0) == (2.5, 4.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")

    class A:
        gpus, steps, warmup = 2, 1, 0

    assert bench.run_reference_arm(A()) is None  # returns before touching the oracle
