"""On-device writeGraph (fb_graph_compile) against the oracle's float64 restatement, and batches of
brains over one topology with per-trial type gains baked into their weights."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(N, seed):
    from flybrain import synth_graph
    g = synth_graph(N, seed)
    rng = np.random.default_rng(seed)
    counts = g.counts.astype(np.float32)
    pre_sign = rng.choice(np.array([-1.0, 0.0, 1.0, 0.5, -0.25], np.float32), N)
    in_scale = rng.uniform(0.05, 1.0, N).astype(np.float32)
    out_scale = rng.lognormal(0, 0.2, N).astype(np.float32)
    sensory = (rng.random(N) < 0.1).astype(np.uint8)
    edge_gain = rng.uniform(0.5, 1.5, g.E).astype(np.float32)
    return g, counts, pre_sign, in_scale, out_scale, sensory, edge_gain


@pytest.mark.parametrize("preInh", [0.0, 0.5])
def test_compile_matches_write_graph(preInh):
    from oracle import oracle as O
    from flybrain import DeviceGraph
    g, counts, pre_sign, in_scale, out_scale, sensory, edge_gain = _inputs(600, 3)
    p = dict(O.DEFAULTS, wSyn=0.3, inhGain=0.8, minSyn=6, preInh=preInh)
    W0, s0 = O.write_graph_f64(g.N, g.indptr, g.indices, counts, pre_sign, p, in_scale=in_scale,
                               sensory_mask=sensory, out_scale=out_scale, edge_gain=edge_gain)
    topo = DeviceGraph(g)
    dg = topo.compile(counts, pre_sign, p, in_scale=in_scale, out_scale=out_scale,
                      sensory_mask=sensory, edge_gain=edge_gain)
    W1, s1 = dg.read()
    assert W1.tobytes() == W0.tobytes()
    assert s1.tobytes() == s0.tobytes()
    # optional inputs absent: factors of one, no mask
    W0, s0 = O.write_graph_f64(g.N, g.indptr, g.indices, counts, pre_sign, p)
    W1, s1 = topo.compile(counts, pre_sign, p).read()
    assert W1.tobytes() == W0.tobytes() and s1.tobytes() == s0.tobytes()


def test_batch_over_shared_topology_with_type_gains():
    """Trials differ in seed, drive set and per-cell-type outgoing gain (outScale)."""
    from oracle import oracle as O
    from flybrain import BrainBatch, DeviceGraph, synth_graph
    N = 3000
    g = synth_graph(N, 9)
    rng = np.random.default_rng(9)
    sign0 = g.sign.astype(np.float32)
    p = dict(O.DEFAULTS, dt=0.1, wSyn=0.275, inhGain=1.0, minSyn=1, adaptInc=0.0, depU=0.0,
             coba=False)
    topo = DeviceGraph(g)
    graphs, oracles = [], []
    for b in range(3):
        gains = rng.lognormal(0, 0.2, 64).astype(np.float32)
        og = gains[g.cell_type]
        dg = topo.compile(g.counts.astype(np.float32), sign0, p, out_scale=og)
        W, s = O.write_graph_f64(N, g.indptr, g.indices, g.counts, sign0, p, out_scale=og)
        graphs.append(dg)
        oracles.append(O.OracleBrain(N, g.indptr, g.indices, W, s, p, seed=10 + b))
    batch = BrainBatch(graphs, p, [10, 11, 12])
    steps = np.array([1500, 900, 1200], np.int32)
    for b in range(3):
        idx = rng.choice(N, int(rng.integers(20, 60)), replace=False).astype(np.int32)
        hz = rng.uniform(50, 250, idx.shape[0])
        batch.set_drive(b, idx, hz)
        for i, h in zip(idx, hz):
            oracles[b].setDriveOne(int(i), float(h))
    batch.record(int(steps.max()), 1 << 20)
    batch.step_uneven(steps)
    for b in range(3):
        c0, r0 = oracles[b].run(int(steps[b]), raster=True)
        c1, r1 = batch.spike_log(b, int(steps[b]), 1 << 20)
        np.testing.assert_array_equal(c1, c0)
        np.testing.assert_array_equal(r1, r0)
        assert oracles[b].v.tobytes() == batch.read("v", b).tobytes()
