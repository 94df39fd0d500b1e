"""Generates the golden brain-step vectors in tests/golden/ from the reference kernel itself.

Run in a container that has the reference tree: it builds the reference src/wasm/lif.c natively
(oracle/Makefile -> oracle/_ref/), drives it through the restated LIFWasm host glue on seeded
scripted scenarios, and saves inputs + the reference's outputs (per-step fired counts, fired
lists in ring order, final state) as .npz fixtures. One case uses an induced subgraph of the
reference's real connectome (public/data/graph_w3.bin), compiled by a restatement of writeGraph.

    python tests/golden/make_golden.py [reference_root]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fly-brain_gb300"))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from flybrain.synth import SYNTH_PARAMS, synth_graph  # noqa: E402
from scenarios import final_state, oracle_runner, run_scenario, save_case  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FLYBRAIN_REFERENCE", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: make_golden.py <reference tree> (or set FLYBRAIN_REFERENCE)")
EXC_SIGN = [0, 1, -1, -1, 1, 1, 1, -1]  # src/lif.js:5


def synth(N, seed):
    g = synth_graph(N, seed)
    return dict(indptr=g.indptr, indices=g.indices, W=g.weights, sign=g.sign)


def real_subgraph(K=600):
    """Breadth-first induced subgraph of the real connectome, in the manner of
    scripts/grad_check.mjs:26-46: start at the best-connected neuron with out-degree < 400."""
    meta = json.load(open(f"{REF}/public/data/meta.json"))
    N = meta["N"]
    raw = np.fromfile(f"{REF}/public/data/graph_w{meta['minWeight']}.bin", dtype=np.uint8)
    hdr = raw[:8].view(np.uint32)
    E = int(hdr[1])
    indptr = raw[8: 8 + (N + 1) * 4].view(np.uint32)
    indices = raw[8 + (N + 1) * 4: 8 + (N + 1) * 4 + E * 4].view(np.uint32)
    weights = raw[8 + (N + 1) * 4 + E * 4: 8 + (N + 1) * 4 + E * 6].view(np.uint16)
    nb = np.fromfile(f"{REF}/public/data/neurons.bin", dtype=np.uint8)
    off = 8 + N * 8 + N * 12 + N * 4 + N * 4 + N * 2
    nt = nb[off: off + N]
    outdeg = np.diff(indptr.astype(np.int64))
    seed = 0
    for i in range(N):
        if outdeg[i] > outdeg[seed] and outdeg[i] < 400:
            seed = i
    pick, pos = [seed], {seed: 0}
    h = 0
    while h < len(pick) and len(pick) < K:
        u = pick[h]
        for j in range(int(indptr[u]), int(indptr[u + 1])):
            if len(pick) >= K:
                break
            q = int(indices[j])
            if q not in pos:
                pos[q] = len(pick)
                pick.append(q)
        h += 1
    n = len(pick)
    ip, ix, wt = [0], [], []
    for a in range(n):
        u = pick[a]
        row = []
        for j in range(int(indptr[u]), int(indptr[u + 1])):
            m = pos.get(int(indices[j]))
            if m is not None:
                row.append((m, int(weights[j])))
        row.sort()
        ix += [m for m, _ in row]
        wt += [w for _, w in row]
        ip.append(len(ix))
    sub_nt = np.array([nt[i] for i in pick], dtype=np.uint8)
    return (n, np.array(ip, dtype=np.uint32), np.array(ix, dtype=np.uint32),
            np.array(wt, dtype=np.uint16), sub_nt)


def cases():
    rng = np.random.default_rng(2024)
    out = []
    # 1. the synthetic current-based model (dt 0.1 ms, 19-slot ring), driven in a shuffled order
    g = synth(2000, 11)
    drv = rng.choice(2000, 40, replace=False)
    out.append(("cuba_synth", g, dict(SYNTH_PARAMS), 7, [
        ["drive", drv.tolist(), [150.0] * 40],
        ["step", 1500],
        ["drive", drv[:10].tolist(), [0.0] * 10],
        ["drive", drv[:5].tolist(), [300.0] * 5],
        ["step", 1500]]))
    # 2. conductance-based reference defaults: adaptation, depression, dt 0.5 ms
    g = synth(1500, 12)
    drv = rng.choice(1500, 60, replace=False)
    out.append(("coba_defaults", g, dict(coba=True), 3, [
        ["drive", drv.tolist(), rng.uniform(20, 200, 60).tolist()],
        ["bias", rng.choice(1500, 30, replace=False).tolist(), 9.0],
        ["thr", rng.choice(1500, 30, replace=False).tolist(), rng.uniform(0, 7, 30).tolist()],
        ["step", 800],
        ["addG", [5, 17, 400], [3.25, 0.5, 7.0], [-1.0, 0.0, -0.25]],
        ["step", 400]]))
    # 3. background events, injections mid-run, a reset, drive removal and re-adding
    g = synth(1000, 13)
    drv = rng.choice(1000, 25, replace=False)
    p = dict(SYNTH_PARAMS, adaptInc=0.5, depU=0.1)
    out.append(("background_inject", g, p, 99, [
        ["background", 40.0, 1.2],
        ["drive", drv.tolist(), [120.0] * 25],
        ["step", 700],
        ["pulse", [1, 2, 3, 999], 4.0],
        ["addG", [10, 10, 11], [1.5, 2.5, -0.75], [0.0, -3.0, 0.0]],
        ["thr", [20, 21], [-3.0, 5.0]],
        ["step", 300],
        ["reset"],
        ["drive", drv[:3].tolist(), [0.0] * 3],
        ["drive", drv[:3].tolist(), [250.0] * 3],
        ["step", 1000]]))
    # 4. presynaptic inhibition of driven neurons (delivery must follow the list order exactly)
    g = synth(800, 14)
    drv = rng.choice(800, 80, replace=False)
    out.append(("presynaptic_inhibition", g, dict(coba=True, preInh=0.5), 5, [
        ["drive", drv.tolist(), [180.0] * 80],
        ["step", 1200]]))
    # 5. induced subgraph of the real connectome, compiled by writeGraph (src/lifwasm.js:14-34)
    if os.path.exists(f"{REF}/public/data/graph_w3.bin"):
        n, ip, ix, cnt, nt = real_subgraph(600)
        p = dict(O.DEFAULTS, coba=True, wSyn=0.3, minSyn=5, adaptInc=0.0, depU=0.0)
        pre_sign = np.array([EXC_SIGN[t] for t in nt], dtype=np.float64)
        W, sign = O.write_graph_f64(n, ip, ix, cnt, pre_sign, p)
        g = dict(indptr=ip, indices=ix, W=W, sign=sign)
        drv = rng.choice(n, 40, replace=False)
        out.append(("real_subgraph", g, p, 1, [
            ["drive", drv.tolist(), [200.0] * 40],
            ["bias", list(range(0, 40)), 9.0],
            ["step", 2000]]))
    return out


def adjoint_fixture():
    """The 600-neuron induced subgraph with its raw synapse counts and transmitter classes, the
    input scripts/grad_check.mjs:45-46 builds for the adjoint check."""
    if not os.path.exists(f"{REF}/public/data/graph_w3.bin"):
        return
    n, ip, ix, cnt, nt = real_subgraph(600)
    os.makedirs(os.path.join(HERE, "adjoint"), exist_ok=True)
    path = os.path.join(HERE, "adjoint", "real_subgraph_counts.npz")
    np.savez_compressed(path, N=np.int32(n), indptr=ip, indices=ix, counts=cnt, nt=nt)
    print(f"real_subgraph_counts: N={n} E={len(ix)} -> {os.path.getsize(path)} bytes")


def flyvis_fixture():
    """A small flyvis-shaped model (630 nodes over 10 hex columns) and three eyes' inputs, run by
    the reference's own fv_step (src/wasm/lif.c:86-93): v after 1, 10 and 100 steps."""
    from flybrain.flyvis import synth_flyvis
    m = synth_flyvis(N=630, seed=5, columns=10)
    rng = np.random.default_rng(55)
    B = 3
    x = np.zeros((B, m["N"]), np.float32)
    for b in range(B):
        for ix in m["inputIdx"].values():
            x[b, ix] = rng.uniform(0, 1, ix.shape[0]).astype(np.float32)
    x[2, :40] = -0.5  # negative drive: nodes fall below zero and stop sending (lif.c:89)
    v = np.tile(m["bias"], (B, 1)).astype(np.float32)
    snaps, done = [], 0
    for upto in (1, 10, 100):
        O.fv_run(m, v, x, upto - done, backend="ref")
        done = upto
        snaps.append(v.copy())
    os.makedirs(os.path.join(HERE, "flyvis"), exist_ok=True)
    path = os.path.join(HERE, "flyvis", "flyvis_synth.npz")
    np.savez_compressed(path, N=np.int32(m["N"]), E=np.int64(m["E"]), indptr=m["indptr"], target=m["target"],
                        weight=m["weight"], bias=m["bias"], tau=m["tau"], dt=np.float64(m["dt"]), x=x,
                        steps=np.array([1, 10, 100], np.int32), v=np.stack(snaps))
    print(f"flyvis_synth: N={m['N']} E={m['E']} -> {os.path.getsize(path)} bytes")


def main():
    O.build(ref=True)
    flyvis_fixture()
    adjoint_fixture()
    for name, g, params, seed, script in cases():
        brain = O.OracleBrain(len(g["sign"]), g["indptr"], g["indices"], g["W"], g["sign"], params,
                              seed=seed, backend="ref")
        blocks = run_scenario(brain, script, oracle_runner)
        st = final_state(brain)
        path = os.path.join(HERE, f"{name}.npz")
        save_case(path, name, g, dict(O.DEFAULTS, **params), seed, script, blocks, st)
        tot = sum(int(c.sum()) for c, _ in blocks)
        print(f"{name}: N={len(g['sign'])} E={len(g['indices'])} spikes={tot} -> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
