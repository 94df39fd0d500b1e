"""Autotuner for the batched launches: times candidate launch shapes on the device, on the
workload itself, and keeps the fastest. Results never depend on the shape (every kernel sums in
a fixed order), so the search only trades speed.

Forward (BrainBatch, grid schedule): resident CTAs per SM (the persistent grid is SMs x that,
512 threads each) x edges per warp work item (32 x item_chunks). The batch keeps stepping from
its current state; each candidate is timed on `steps` steps (the device-side launch time), the
best of `repeats`.

Adjoint (DiffBatch): the checkpoint interval K (a short K keeps a replayed segment's arena in L2
for small batches; a long one makes fewer, longer segments), then the blocks per member of the
thread-per-neuron kernels, then of the warp-per-arrival kernels (coordinate descent: each knob
searched with the others at their best so far), each candidate timed on a recorded forward plus
backward of `steps` steps with the caller's loss gradient.

Choices are cached per (workload key, device) in a JSON file (FLYBRAIN_TUNE_CACHE, default
~/.cache/flybrain/tune.json); a cache hit skips the search.
"""
from __future__ import annotations

import json
import os
import time

from . import _native as nat


def _cache_path() -> str:
    return os.environ.get("FLYBRAIN_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "flybrain",
                                                                 "tune.json")


def _device() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001 - the key only needs to be stable
        return "cuda:0"


def _load() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value: dict) -> None:
    d = _load()
    d[key] = value
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs a search next time


def _sync():
    import torch
    torch.cuda.synchronize()


def tune_brains(batch, steps: int = 100, blocks_per_sm=None, item_chunks=(1, 2, 4, 8), repeats: int = 2,
                key: str | None = None, use_cache: bool = True) -> dict:
    """Search the grid schedule's launch shape for `batch` (a BrainBatch) and apply the fastest.
    Returns {"blocks_per_sm", "item_chunks", "ms_per_step", "table": [...], "cached"}."""
    cur = batch.tuning()
    bps = list(blocks_per_sm or range(1, cur["max_blocks_per_sm"] + 1))
    key = "brains|" + (key or f"B={batch.B}") + "|" + _device()
    if use_cache:
        hit = _load().get(key)
        if hit and hit["blocks_per_sm"] <= cur["max_blocks_per_sm"]:
            batch.set_tuning(hit["blocks_per_sm"], hit["item_chunks"])
            return dict(hit, cached=True)
    batch.set_schedule(nat.FB_SCHEDULE_GRID)
    table = []
    try:
        batch.step(steps)  # warm-up at the current shape
        for b in bps:
            for c in item_chunks:
                batch.set_tuning(b, c)
                best = float("inf")
                for _ in range(max(1, repeats)):
                    batch.step(steps)
                    best = min(best, batch.last_ms())
                table.append(dict(blocks_per_sm=b, item_chunks=c, ms_per_step=best / steps))
    finally:
        batch.set_schedule(nat.FB_SCHEDULE_AUTO)
    win = min(table, key=lambda r: r["ms_per_step"])
    batch.set_tuning(win["blocks_per_sm"], win["item_chunks"])
    out = dict(win, table=table)
    if use_cache:
        _store(key, out)
    return dict(out, cached=False)


def tune_diff(batch, steps, seeds, dLs, readouts=None, Ks=(25, 50, 100, 200), neuron_blocks=None,
              arrival_blocks=None, key: str | None = None, use_cache: bool = True) -> dict:
    """Search K and the per-step kernels' launch shape for `batch` (a DiffBatch) and apply the
    fastest: batch.p["checkpoint"] = K and the batch's tuning. steps/seeds as
    DiffBatch.forward takes them; dLs/readouts as DiffBatch.backward takes them. Candidates are
    timed with step launches (a captured pass's first run would include its capture); the batch's
    launch mode is restored afterwards.
    Returns {"checkpoint", "neuron_blocks", "arrival_blocks", "s", "table", "cached"}."""
    key = "diff|" + (key or f"B={batch.B}|N={sum(batch.N)}") + "|" + _device()
    if use_cache:
        hit = _load().get(key)
        if hit:
            batch.p["checkpoint"] = hit["checkpoint"]
            batch.set_tuning(hit["neuron_blocks"], hit["arrival_blocks"])
            return dict(hit, cached=True)
    table = []
    mode = dict(getattr(batch, "tuning", None) or {}).get("step_launches", False)

    def run(K, nb, ab):
        batch.set_tuning(nb, ab, step_launches=True)
        _sync()
        t0 = time.perf_counter()
        batch.forward(steps, seeds, record=True, counts=False, checkpoint=K)
        batch.backward(dLs, readouts, edge=False)
        _sync()
        s = time.perf_counter() - t0
        table.append(dict(checkpoint=K, neuron_blocks=nb, arrival_blocks=ab, s=s))
        return s

    # the defaults, for scale and a warm-up
    tiles = max((n + 255) // 256 for n in batch.N)
    nb_opts = list(neuron_blocks or sorted({max(1, tiles // d) for d in (1, 2, 4, 8, 16, 32)}))
    ab_opts = list(arrival_blocks or (2, 4, 8, 16, 32, 64))
    K0 = int(batch.p.get("checkpoint", 100))
    run(max(list(Ks) + [K0]), 0, 0)  # warm-up at the longest K: the replay arena is allocated once
    best = dict(checkpoint=K0, neuron_blocks=0, arrival_blocks=0, s=run(K0, 0, 0))
    for K in sorted(set(Ks) - {K0}, reverse=True):
        s = run(K, 0, 0)
        if s < best["s"]:
            best = dict(best, checkpoint=K, s=s)
    for nb in nb_opts:
        s = run(best["checkpoint"], nb, best["arrival_blocks"])
        if s < best["s"]:
            best = dict(best, neuron_blocks=nb, s=s)
    for ab in ab_opts:
        s = run(best["checkpoint"], best["neuron_blocks"], ab)
        if s < best["s"]:
            best = dict(best, arrival_blocks=ab, s=s)
    batch.p["checkpoint"] = best["checkpoint"]
    batch.set_tuning(best["neuron_blocks"], best["arrival_blocks"], step_launches=mode)
    out = dict(best, table=table)
    if use_cache:
        _store(key, out)
    return dict(out, cached=False)
