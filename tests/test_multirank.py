"""Host logic of the multi-rank benchmark, on CPU with the gloo backend and
two ranks: each rank evaluates its own replica, the job time is the slowest
rank's, and throughput sums the ranks' interactions."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        t = bench.max_over_ranks(1.0 + rank, world, device="cpu")
        v = bench.job_throughput(10 ** 9, 2, t, world)
        out[rank] = (t, v)
    finally:
        dist.destroy_process_group()


def test_two_rank_replica_aggregation():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1]
    t, v = res[0]
    assert t == 2.0  # the slowest rank bounds the job
    assert v == pytest.approx(2 * 1e9 * 2 / 2.0 / 1e9)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(5 * 10 ** 9, 1, 1.0, 1) == pytest.approx(5.0)
