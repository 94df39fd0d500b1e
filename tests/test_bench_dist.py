"""The replica path of bench.py (one process per GPU, no data-path collective): its barrier and
its whole-job reduction (events summed over ranks, time = the slowest rank's) on world_size-2
gloo process groups on the CPU; and the reference arm's rank > 0 behaviour (exit without work)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), FB_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init()
    try:
        bench.barrier(w)
        events = 1000.0 * (rank + 1)
        secs = 2.0 + rank
        out = dict(rank=r, world=w, mx=bench.max_over_ranks(secs, w), sm=bench.sum_over_ranks(events, w),
                   thr=bench.replica_throughput(events, secs, w))
        bench.barrier(w)
        q.put(out)
    finally:
        dist.destroy_process_group()


def test_replica_reduction_world2():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for o in res:
        assert o["world"] == 2
        assert o["mx"] == 3.0          # the slowest rank's time
        assert o["sm"] == 3000.0       # 1000 + 2000 events
        assert o["thr"] == 1000.0      # 3000 events / 3 s


def test_single_process_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5, 1) == 2.5
    assert bench.sum_over_ranks(7.0, 1) == 7.0
    assert bench.replica_throughput(10.0, 2.0, 1) == 5.0
