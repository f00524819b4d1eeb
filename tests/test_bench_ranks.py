"""The multi-rank path of bench.py on CPU: two gloo ranks.

Each rank times its own frames (weak scaling, no data-path collective); the
reported time is the slowest rank's (an all-reduce MAX of one number) and
the rate counts the frames of all ranks.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 25.0 * rank  # rank 1 is the slower one
        ms_max = bench.max_over_ranks(ms, dist, "cpu")
        value = bench.whole_job_rate(world, 2_000_000, 10, ms_max)
        out.put((rank, ms_max, value, bench.rank_seed(rank)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, v0, s0), (r1, m1, v1, s1) = results
    assert m0 == m1 == 125.0
    assert v0 == v1 == pytest.approx(2 * 2_000_000 * 10 / 0.125)
    assert s0 != s1  # each rank draws its own frames


def test_single_rank_needs_no_collective():
    import bench
    assert bench.max_over_ranks(42.0, None, "cpu") == 42.0
    assert bench.whole_job_rate(1, 1000, 4, 2.0) == pytest.approx(2e6)
