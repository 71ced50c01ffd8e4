"""Replicas across ranks, as bench.py runs them under torchrun (one process
per GPU, every rank its own beams, no data exchanged): the only collectives
are the slowest rank's time (max) and the units all ranks processed (sum).
Checked with two gloo ranks on the CPU; the reference arm's non-zero ranks
exit without work."""
import os
import socket
import sys
import types
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, units, seconds, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench

    rate, slowest = bench.job_rate(dist, units[rank], seconds[rank], device="cpu")
    q.put((rank, rate, slowest))
    dist.barrier()
    dist.destroy_process_group()


def _run_ranks(units, seconds):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, len(units), port, units, seconds, q)) for r in range(len(units))]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def test_job_rate_two_ranks():
    # rank 0: 10 beam-seconds in 1 s, rank 1: 20 in 2 s -> 30 over the slowest 2 s
    out = _run_ranks([10.0, 20.0], [1.0, 2.0])
    assert [r for r, _, _ in out] == [0, 1]
    for _, rate, slowest in out:
        assert rate == pytest.approx(15.0) and slowest == pytest.approx(2.0)


def test_job_rate_uneven_ranks():
    out = _run_ranks([7.0, 7.0], [0.5, 0.25])
    for _, rate, slowest in out:
        assert rate == pytest.approx(28.0) and slowest == pytest.approx(0.5)


def test_job_rate_single_process():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.job_rate(None, 12.0, 4.0) == (3.0, 4.0)


def test_reference_arm_nonzero_rank_does_no_work(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    a = types.SimpleNamespace(workload="full", steps=1, warmup=3)
    assert bench.run_reference(a, rank=1, world=2) is None
    assert capsys.readouterr().out == ""
