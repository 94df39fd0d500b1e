"""Seeded synthetic connectome-shaped graphs and drive sets.

The workloads are synthetic stand-ins for the reference's connectome (public/data/graph_w3.bin,
165,122 neurons): the same CSR layout and value types, with shapes drawn from a fixed recipe.

Graph recipe (per presynaptic neuron i):
  * out-degree  = clip(round(lognormal(mu=3.5, sigma=1.2)), 1, 5000)
  * targets     = 80% uniform within i +- N/50 (mod N), 20% uniform over all neurons;
                  duplicate (pre, post) pairs are merged, each row is sorted by target
  * count       = 5 + Geometric(p=0.3) failures (synapses per connection)
  * sign        = +1 with probability 0.6, else -1 (per presynaptic neuron)
  * weight      = float32(count * 0.275) computed in float64 and rounded once, as writeGraph
                  (src/lifwasm.js:31) rounds its double-precision product once
The compiled arrays are what the brain step consumes: indptr u32[N+1], indices u32[E],
weights f32[E], sign f32[N] (src/lifwasm.js:14-34 layout).
"""
from __future__ import annotations

import numpy as np

W_PER_SYNAPSE = 0.275


class Graph:
    """A compiled CSR graph: indptr, indices, weights (f32) and per-neuron sign (f32)."""

    def __init__(self, N, indptr, indices, weights, sign, counts=None, cell_type=None):
        self.N = int(N)
        self.indptr = np.ascontiguousarray(indptr, dtype=np.uint32)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32)
        self.weights = np.ascontiguousarray(weights, dtype=np.float32)
        self.sign = np.ascontiguousarray(sign, dtype=np.float32)
        self.counts = None if counts is None else np.ascontiguousarray(counts, dtype=np.uint16)
        self.cell_type = None if cell_type is None else np.ascontiguousarray(cell_type, dtype=np.uint8)

    @property
    def E(self) -> int:
        return int(self.indices.shape[0])

    def outdeg(self) -> np.ndarray:
        return np.diff(self.indptr.astype(np.int64))


def synth_graph(N: int, seed: int, mu: float = 3.5, sigma: float = 1.2, max_deg: int = 5000,
                local_frac: float = 0.8, exc_frac: float = 0.6, geo_p: float = 0.3,
                base_count: int = 5, n_types: int = 64) -> Graph:
    """Seeded connectome-shaped CSR graph (recipe in the module docstring)."""
    rng = np.random.default_rng(seed)
    deg = np.clip(np.round(rng.lognormal(mu, sigma, N)), 1, max_deg).astype(np.int64)
    pre = np.repeat(np.arange(N, dtype=np.int64), deg)
    tot = pre.shape[0]
    half = max(1, N // 50)
    local = rng.random(tot) < local_frac
    near = (pre + rng.integers(-half, half + 1, tot)) % N
    far = rng.integers(0, N, tot)
    post = np.where(local, near, far)
    key = pre * N + post
    key.sort()
    key = key[np.concatenate(([True], key[1:] != key[:-1]))]  # merges duplicates; sorted by (pre, post)
    pre = key // N
    post = key % N
    E = key.shape[0]
    indptr = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(np.bincount(pre, minlength=N), out=indptr[1:])
    counts = base_count + rng.geometric(geo_p, E) - 1
    sign = np.where(rng.random(N) < exc_frac, 1.0, -1.0).astype(np.float32)
    weights = (counts.astype(np.float64) * W_PER_SYNAPSE).astype(np.float32)
    cell_type = rng.integers(0, n_types, N).astype(np.uint8)
    return Graph(N, indptr.astype(np.uint32), post.astype(np.uint32), weights, sign,
                 counts.astype(np.uint16), cell_type)


def drive_set(N: int, n_driven: int, seed: int, lo_hz: float, hi_hz: float):
    """Seeded sensory drive: n_driven distinct neurons (ascending) with rates uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(N, size=n_driven, replace=False)).astype(np.int32)
    if lo_hz == hi_hz:
        hz = np.full(n_driven, lo_hz, dtype=np.float64)
    else:
        hz = rng.uniform(lo_hz, hi_hz, n_driven)
    return idx, hz


# LIF parameters of the synthetic workloads (CUBA, no adaptation or depression, no background).
SYNTH_PARAMS = dict(
    dt=0.1, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
    wSyn=1.0, traceTau=30.0, adaptInc=0.0, adaptTau=100.0, depU=0.0, depTau=200.0, coba=False,
    eExc=0.0, eInh=-70.0, preInh=0.0, bgRate=0.0, bgAmp=0.0,
)


def workload(name: str, seed: int = 1):
    """(graph, drive index, drive Hz, steps) of a named synthetic workload.

    small: N=20,000, 150 Hz into 1% of neurons, 10,000 steps (1,000 ms at dt 0.1 ms).
    full : N=165,122, 2,000 neurons at U(100, 200) Hz, 20,000 steps (2,000 ms).
    """
    if name == "small":
        N = 20000
        g = synth_graph(N, seed)
        idx, hz = drive_set(N, N // 100, seed + 1000, 150.0, 150.0)
        return g, idx, hz, 10000
    if name == "full":
        N = 165122
        g = synth_graph(N, seed)
        idx, hz = drive_set(N, 2000, seed + 1000, 100.0, 200.0)
        return g, idx, hz, 20000
    raise ValueError(f"unknown workload {name!r}")
