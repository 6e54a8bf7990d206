"""The multi-rank path of bench.py on CPU: N replicas (one per GPU on a node; here gloo
processes on 127.0.0.1) time the same step, the job takes the slowest rank's time and counts
the bases of every rank (weak scaling, no data-path collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        q.put((rank, ms, bench.job_gbases_per_s(1_000_000_000, world, ms)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_count_all_bases():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    # both ranks see the slower rank's 15 ms; 2 x 1 Gbases in 15 ms = 133.3 Gbases/s
    assert [(r, ms) for r, ms, _ in got] == [(0, 15.0), (1, 15.0)]
    assert all(abs(v - 2e9 / 15e-3 / 1e9) < 1e-6 for _, _, v in got)


def test_single_rank_keeps_its_own_time():
    import bench

    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.job_gbases_per_s(1_000_000_000, 1, 50.0) == pytest.approx(20.0)
