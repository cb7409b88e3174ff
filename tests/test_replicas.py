"""Multi-GPU runs are replicas only (independent mesh pairs, no collective
on the data path): the bench's N-rank logic, on CPU with gloo. Each rank
times its own replica; the job's time is the slowest rank's; the value is
all ranks' units over that time; only rank 0 reports."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    r, w, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    times = bench.max_over_ranks([10.0 + 5 * rank, 7.0 - rank], dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, local, times, bench.replicas_value(30, w, times[0])))


@pytest.mark.parametrize("world", [2, 3])
def test_max_over_ranks_and_value_with_gloo(world):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = 10.0 + 5 * (world - 1)
    for r, (rank, w, local, times, value) in enumerate(out):
        assert (rank, w, local) == (r, world, r)
        assert times == [slowest, 7.0]  # every rank sees the max over ranks
        assert value == pytest.approx(30 * world / (slowest / 1e3))


def test_single_process_needs_no_group():
    import bench

    assert bench.max_over_ranks([3.0, 4.0], None, "cpu") == [3.0, 4.0]
    assert bench.replicas_value(100, 1, 50.0) == pytest.approx(2000.0)
