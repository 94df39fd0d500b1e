"""Scripted brain scenarios, replayed identically on the oracle, the reference build and the GPU.

A scenario is a graph, params, a seed and a list of operations in the LIFWasm vocabulary
(src/lifwasm.js:69-85): drive/bias/thr/addG/pulse/background/reset, and ("step", n) blocks.
`run_scenario` returns, for every step block, the per-step fired counts and the concatenated
fired lists, plus the final per-neuron state.
"""
from __future__ import annotations

import json

import numpy as np

STATE_FIELDS = ("v", "gE", "gI", "refr", "trace", "adapt", "res", "spikeCount")


def apply_op(brain, op):
    kind = op[0]
    if kind == "drive":
        for i, hz in zip(op[1], op[2]):
            brain.setDriveOne(int(i), float(hz))
    elif kind == "bias":
        brain.setBias([int(i) for i in op[1]], float(op[2]))
    elif kind == "thr":
        for i, mv in zip(op[1], op[2]):
            brain.setThr(int(i), float(mv))
    elif kind == "addG":
        for i, e, ii in zip(op[1], op[2], op[3]):
            brain.addG(int(i), float(e), float(ii))
    elif kind == "pulse":
        brain.pulse([int(i) for i in op[1]], float(op[2]))
    elif kind == "background":
        brain.setBackground(float(op[1]), float(op[2]))
    elif kind == "reset":
        brain.reset()
    else:
        raise ValueError(kind)


def run_scenario(brain, script, runner):
    """runner(brain, n) -> (counts[n], raster) advances n steps and returns what they fired."""
    blocks = []
    for op in script:
        if op[0] == "step":
            counts, raster = runner(brain, int(op[1]))
            blocks.append((np.asarray(counts, dtype=np.int32), np.asarray(raster, dtype=np.int32)))
        else:
            apply_op(brain, op)
    return blocks


def oracle_runner(brain, n):
    return brain.run(n, raster=True)


def final_state(brain):
    return {k: np.array(getattr(brain, k)).copy() for k in STATE_FIELDS}


def save_case(path, name, graph, params, seed, script, blocks, state):
    arrs = dict(indptr=graph["indptr"], indices=graph["indices"], W=graph["W"], sign=graph["sign"])
    for k, (c, r) in enumerate(blocks):
        arrs[f"counts{k}"] = c
        arrs[f"raster{k}"] = r
    for k, v in state.items():
        arrs[f"state_{k}"] = v
    meta = dict(name=name, N=int(len(graph["sign"])), params=params, seed=int(seed),
                script=script, nblocks=len(blocks))
    arrs["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(path, **arrs)


def load_case(path):
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    graph = dict(indptr=z["indptr"], indices=z["indices"], W=z["W"], sign=z["sign"])
    blocks = [(z[f"counts{k}"], z[f"raster{k}"]) for k in range(meta["nblocks"])]
    state = {k: z[f"state_{k}"] for k in STATE_FIELDS}
    return meta, graph, blocks, state
