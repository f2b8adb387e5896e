"""The benchmark's multi-rank path on CPU: two gloo ranks (replicas) reduce
their timings to the slowest rank's, and the whole-job rate counts every
rank's input.  No GPU and no collective on the data path is involved."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 10 + r ms on device and 20 - r ms end to end
        got = bench.max_over_ranks([10.0 + rank, 20.0 - rank], world, "cpu")
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res[0] == res[1] == [11.0, 20.0]


def test_whole_job_rate_counts_every_replica():
    sys.path.insert(0, ROOT)
    import bench
    one = bench.whole_job_gbs(100e6, 10, 1, 20.0)
    two = bench.whole_job_gbs(100e6, 10, 2, 20.0)
    assert one == pytest.approx(50.0)
    assert two == pytest.approx(2 * one)
    assert bench.max_over_ranks([3.0, 4.0], 1, None) == [3.0, 4.0]
