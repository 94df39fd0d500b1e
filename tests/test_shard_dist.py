"""Trials split over ranks (flybrain.shard) and the ordered cross-rank gradient sum, on gloo
process groups on the CPU (world sizes 2 and 3): every trial is run by exactly one rank, and the
sum of per-trial arrays in global trial order is bit-identical to one process adding them in a
loop, whatever the number of ranks. The arrays span many orders of magnitude, so any other
summation order gives a different float64 result (checked)."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
B, LEN = 11, 4096


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def per_trial(b):
    """Trial b's synthetic per-edge gradient (float32, wide dynamic range, both signs)."""
    rng = np.random.default_rng(100 + b)
    return (rng.standard_normal(LEN) * 10.0 ** rng.uniform(-8, 8, LEN)).astype(np.float32)


def in_order_sum():
    acc = torch.from_numpy(per_trial(0)).to(torch.float64)
    for b in range(1, B):
        acc = acc + torch.from_numpy(per_trial(b)).to(torch.float64)
    return acc.numpy()


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.path.join(ROOT, "fly-brain_gb300"))
    from flybrain.shard import ordered_sum, trials_of_rank
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = trials_of_rank(B, rank, world, "blocks")
        arrays = [torch.from_numpy(per_trial(int(b))) for b in mine]
        out = ordered_sum(arrays, B, rank, world, (LEN,))
        q.put((rank, mine.tolist(), trials_of_rank(B, rank, world).tolist(), out.numpy().tobytes()))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_ordered_sum_equals_the_one_process_sum(world):
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = in_order_sum()
    blocks = [r[1] for r in res]
    inter = [r[2] for r in res]
    assert sorted(sum(blocks, [])) == list(range(B)) and sum(blocks, []) == list(range(B))
    assert sorted(sum(inter, [])) == list(range(B))
    for rank, _, _, out in res:
        assert np.frombuffer(out, np.float64).tobytes() == want.tobytes(), rank
    # the data is order-sensitive: the reverse order does not give the same bits
    rev = torch.from_numpy(per_trial(B - 1)).to(torch.float64)
    for b in range(B - 2, -1, -1):
        rev = rev + torch.from_numpy(per_trial(b)).to(torch.float64)
    assert rev.numpy().tobytes() != want.tobytes()


def test_trial_assignment():
    sys.path.insert(0, os.path.join(ROOT, "fly-brain_gb300"))
    from flybrain.shard import trials_of_rank
    for n in (0, 1, 7, 256):
        for w in (1, 2, 3, 8):
            for mode in ("interleaved", "blocks"):
                parts = [trials_of_rank(n, r, w, mode).tolist() for r in range(w)]
                flat = sum(parts, [])
                assert sorted(flat) == list(range(n))
                if mode == "blocks":
                    assert flat == list(range(n))
                    assert max(map(len, parts)) - min(map(len, parts)) <= 1
    assert trials_of_rank(10, 1, 4).tolist() == [1, 5, 9]
    with pytest.raises(ValueError):
        trials_of_rank(4, 2, 2)
