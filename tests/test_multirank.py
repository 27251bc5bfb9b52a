"""The benchmark's multi-rank path on CPU with two gloo ranks (torchrun launches one rank per
GPU; the ranks are independent replicas with no data-path collective): the timing is the
slowest rank's, the rate is the whole job's, and the reference arm runs on rank 0 alone."""

import io
import contextlib
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.0 + rank, world, "cpu")  # rank 1 is the slower one
        out[rank] = (t, bench.whole_job_rate(world, 3, 10, t))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_is_the_slowest_rank():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork from a threaded process
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0
    assert res[0][1] == res[1][1] == pytest.approx(2 * 3 * 10 / 2.0)


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(1.5, 1, "cpu") == 1.5
    assert bench.whole_job_rate(1, 256, 10, 1.0) == 2560.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    args = argparse.Namespace(config="baroclinic3_128", steps=1, warmup=0, gpus=2)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ""  # rank 1 exits without work or output
