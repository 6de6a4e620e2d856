"""The bench's multi-rank host logic on CPU (gloo, two ranks): one process per GPU, each its own replica, so the
job's time is the slowest rank's and the job's throughput the units of all ranks over that time; the reference
arm runs on rank 0 alone, and the other ranks leave without work."""
import os
import socket
import time

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, _ = bench.dist_env()
    ms = 10.0 + 5.0 * r                       # rank 1 is the slow one
    slowest = bench.max_over_ranks(ms, w)
    thr = bench.job_throughput(20, slowest, w)
    skipped = None
    if r != 0:
        # the reference arm: ranks other than 0 return at once, without work or output
        t = time.perf_counter()
        bench.run_reference(None)           # rank != 0 returns before it reads its arguments
        skipped = time.perf_counter() - t
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, slowest, thr, skipped))


def test_two_ranks_take_the_slowest_rank_and_sum_the_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[:2] for o in out] == [(0, 2), (1, 2)]
    for _, _, slowest, thr, _ in out:
        assert slowest == 15.0
        assert thr == pytest.approx(20 * 2 / 0.015)
    assert out[1][4] is not None and out[1][4] < 1.0


def test_one_rank_is_its_own_time():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.job_throughput(10, 500.0, 1) == pytest.approx(20.0)
