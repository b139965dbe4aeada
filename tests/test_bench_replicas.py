"""The multi-GPU form of bench.py is replicas: each rank runs the whole
workload on its own GPU and only the timings cross ranks (max over ranks,
whole-job rate = ranks x units per step x steps / slowest time).  This checks
that host logic with two gloo ranks on the CPU."""
import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        # rank r was slower on the first value and faster on the second
        vals = bench.reduce_max([10.0 + rank, 5.0 - rank, 7.0], dist, "cpu")
        out[rank] = vals
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_two_gloo_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        got = dict(out)
    assert got[0] == got[1] == [11.0, 5.0, 7.0]


def test_single_rank_is_unchanged_and_rate_is_whole_job():
    import bench
    assert bench.reduce_max([3.0, 4.0], None, "cpu") == [3.0, 4.0]
    # 2 replicas x 1e6 units per step x 100 steps in 50 ms -> 4e9 units/s
    assert bench.replica_rate(2, 1_000_000, 100, 50.0) == pytest.approx(4e9)
