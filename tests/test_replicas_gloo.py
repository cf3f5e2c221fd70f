"""The host-side logic of multi-GPU runs (replicas, one process per GPU) on
CPU: two gloo ranks over 127.0.0.1."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from yael_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank "timed" a different duration; the job's time is the slowest
        t = replicas.max_over_ranks(1.5 + rank, dist)
        rate = replicas.whole_job_rate(10_000, t, world)
        seed = replicas.query_seed(rank)
        out[rank] = (t, rate, seed)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_replica_aggregation():
    world = 2
    mgr = mp.get_context("spawn").Manager()  # no fork of this (threaded) process
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 2.5          # both ranks see the slowest time
    assert out[0][1] == out[1][1] == 2 * 10_000 / 2.5  # weak scaling: all ranks' units
    assert out[0][2] == 2 and out[1][2] == 1002    # distinct query sets per rank


def test_single_process_helpers():
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.whole_job_rate(100, 2.0, 1) == 50.0
    with pytest.raises(ValueError):
        replicas.whole_job_rate(1, 0.0, 1)
