"""The bench's N-replica aggregation (torchrun, one process per GPU) on CPU
with the gloo backend and two ranks: the job's time is the slowest rank's
(max over ranks) and its value counts every rank's work.  The GPU run
itself has one GPU here; this covers the host logic of N > 1."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = 2.0 + 3.0 * rank                       # rank 1 is the slow one
        got = bench.max_over_ranks(ms, dist, device="cpu")
        out.put((rank, got, bench.whole_job_gflops(world, 1_000_000, got)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [5.0, 5.0]
    # 2 ranks x 2 MFLOP in 5 ms
    assert all(abs(r[2] - 2 * 2.0 * 1_000_000 / (5.0 * 1e6)) < 1e-12 for r in res)


def test_one_rank_is_itself():
    import bench
    assert bench.max_over_ranks(7.5, None) == 7.5
    assert bench.whole_job_gflops(1, 500_000_000, 1000.0) == pytest.approx(1.0)
