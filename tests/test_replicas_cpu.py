"""Multi-GPU form of the bench is replicas only: each rank registers its own
pairs, the slowest rank's time sets the whole-job time, and the job's rate
is every rank's units over that time.  The host logic runs here as two
`gloo` ranks on CPU (no GPU, no data-path collective)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "measured" (10 + r) ms device time and (20 - r) ms wall time
        ms, wall = bench.max_over_ranks([10.0 + rank, 20.0 - rank], dist, "cpu")
        out.put((rank, ms, wall, bench.job_rate(world, 5, ms), bench.replica_seeds(rank, 3)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_bench():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, wall, rate, seeds in got:
        assert ms == 11.0 and wall == 20.0          # max over both ranks, element-wise
        assert rate == pytest.approx(2 * 5 / 0.011)  # all ranks' units over the slowest time
    assert set(got[0][4]).isdisjoint(got[1][4])      # each replica has its own pairs


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3.0, 4.0], None, "cpu") == [3.0, 4.0]
    assert bench.job_rate(1, 10, 100.0) == pytest.approx(100.0)
