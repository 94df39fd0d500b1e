"""The batched ensemble: many independent flies (trials) sharing one connectome topology, as
src/brainsetup.js:10-28 gives every fly of a multi-fly scene its own state block over one
read-only graph (src/lifwasm.js:90-98).

ensemble_spec draws every trial's inputs from one seeded stream: its outgoing per-cell-type gains
(lognormal(0, 0.2) over 64 types, compiled into its weights as writeGraph's outScale,
src/lifwasm.js:14-34), its generator seed, its duration U(200, 2000) ms and its drive set of
U{500..4000} neurons at U(50, 250) Hz. The draws do not depend on how the trials are later split,
so trial b is the same fly whichever process or GPU runs it.

Over several GPUs, rank r of `world` runs the trials b = r, r + world, ... (flybrain.shard,
interleaved): the ensemble's only parallel axis, with no exchange between ranks.
"""
from __future__ import annotations

import numpy as np

from .shard import trials_of_rank  # noqa: F401  (the ensemble's split over ranks)

N_TYPES = 64


def ensemble_spec(N: int, n_trials: int, seed: int = 7, dt: float = 0.1) -> dict:
    """Per-trial inputs of the ensemble over an N-neuron graph (host arrays, deterministic)."""
    rng = np.random.default_rng(seed)
    gains = [rng.lognormal(0.0, 0.2, N_TYPES).astype(np.float32) for _ in range(n_trials)]
    seeds = rng.integers(1, 1 << 30, n_trials)
    steps = np.round(rng.uniform(200.0, 2000.0, n_trials) / dt).astype(np.int32)
    drives = []
    for _ in range(n_trials):
        nd = int(rng.integers(500, 4001))
        idx = np.sort(rng.choice(N, nd, replace=False)).astype(np.int32)
        drives.append((idx, rng.uniform(50.0, 250.0, nd)))
    return dict(n_trials=n_trials, gains=gains, seeds=np.asarray(seeds, np.int64), steps=steps, drives=drives)


def build_ensemble(g, spec: dict, params: dict, trials=None):
    """A BrainBatch of the chosen trials (all by default) over graph g's topology: each trial's
    weights compiled on the device with its type gains, its seed and drive set applied.
    Returns (batch, per-trial compiled DeviceGraphs, trial ids)."""
    import torch

    from .brain import BrainBatch, DeviceGraph

    trials = np.arange(spec["n_trials"]) if trials is None else np.asarray(trials, np.int64)
    topo = DeviceGraph(g)
    counts = torch.from_numpy(g.counts.astype(np.float32)).cuda()
    sign = torch.from_numpy(g.sign.astype(np.float32)).cuda()
    ctype = torch.from_numpy(g.cell_type.astype(np.int64)).cuda()
    graphs = []
    for b in trials.tolist():
        gains = torch.from_numpy(spec["gains"][b]).cuda()
        graphs.append(topo.compile(counts, sign, params, out_scale=gains[ctype].contiguous()))
    torch.cuda.synchronize()
    batch = BrainBatch(graphs, params, spec["seeds"][trials])
    for k, b in enumerate(trials.tolist()):
        idx, hz = spec["drives"][b]
        batch.set_drive(k, idx, hz)
    return batch, graphs, trials
