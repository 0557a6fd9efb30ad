"""The N > 1 path of bench.py without a GPU: two ranks over gloo on CPU
(127.0.0.1).  Each replica times its own image; the job's step time is the
slowest rank's, its rate counts every rank's pixels, and the reference arm
does its work on rank 0 only."""
import argparse
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, step_ms, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        m = bench.max_over_ranks(step_ms[rank], dist, torch.device("cpu"))
        q.put((rank, m, bench.job_rate_mpix_s(world, 8_294_400, m)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_step():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    step_ms = [1.25, 1.75]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, step_ms, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for _, m, rate in got:
        assert m == 1.75
        assert rate == pytest.approx(2 * 8_294_400 / 1.75e-3 / 1e6)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(2.5, None, None) == 2.5
    assert bench.job_rate_mpix_s(1, 1_000_000, 1.0) == pytest.approx(1000.0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    import bench
    args = argparse.Namespace(warmup=3, steps=2, ref_side=64, gpus=2)
    assert bench.run_reference(args, 1) is None
    assert capsys.readouterr().out == ""
