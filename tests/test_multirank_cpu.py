"""CPU: the N>1 replica path of bench.py over torch.distributed gloo with two
ranks -- the max-over-ranks timing and the whole-job aggregate."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, results):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_seconds = 1.0 + rank  # rank 1 is the slow one
        results[rank] = (bench.max_over_ranks(local_seconds, "cpu"),
                         bench.aggregate_rate(1000.0, local_seconds, "cpu"))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_aggregation():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        results = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        for r in range(2):
            mx, rate = results[r]
            assert mx == 2.0                      # slowest rank's time on every rank
            assert rate == pytest.approx(1000.0)  # 2 ranks x 1000 units / 2 s


def test_single_rank_identity():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.aggregate_rate(10.0, 2.0, "cpu") == 5.0
