"""Rows that name one target more than once. lif.c delivers every edge of a row in row order
(src/wasm/lif.c:40-42), so an arrival adds its contributions to a repeated target one after the
other; float addition is not associative, so the order shows in the bits. The library keys each
contribution by (arrival rank, repeat index within the row) and the adjoint orders by (arrival,
edge id); here both forward kernels and the adjoint run a graph whose rows repeat targets (with
different weights) bit for bit against the oracle, and a row naming a target more than four times
is refused."""
import numpy as np
import pytest

from test_lagged_gpu import assert_same_as_oracle, lagged_chunks
from test_step_gpu import gpu_multistep, gpu_stepwise

pytestmark = pytest.mark.gpu


def repeated_graph(N=3000, seed=17, frac=0.2):
    """A synthetic graph where a fraction of the rows repeat some of their targets 1-3 extra
    times, each copy with its own synapse count, inserted at random places in the row."""
    from flybrain.synth import Graph, synth_graph
    g = synth_graph(N, seed)
    rng = np.random.default_rng(seed)
    indptr, indices, counts = [0], [], []
    for r in range(N):
        lo, hi = int(g.indptr[r]), int(g.indptr[r + 1])
        row_t = g.indices[lo:hi].tolist()
        row_c = g.counts[lo:hi].tolist()
        if hi > lo and rng.random() < frac:
            for t in rng.choice(row_t, min(3, len(row_t)), replace=False).tolist():
                for _ in range(int(rng.integers(1, 4))):
                    at = int(rng.integers(0, len(row_t) + 1))
                    row_t.insert(at, t)
                    row_c.insert(at, float(5 + rng.geometric(0.3) - 1))
        indices += row_t
        counts += row_c
        indptr.append(len(indices))
    indptr = np.asarray(indptr, np.uint32)
    indices = np.asarray(indices, np.uint32)
    counts = np.asarray(counts, np.float32)
    weights = (counts.astype(np.float64) * 0.275).astype(np.float32)
    return Graph(N=N, indptr=indptr, indices=indices, weights=weights, sign=g.sign.copy(), counts=counts,
                 cell_type=g.cell_type)


def _pair(g, p, seed, nd=60, rate=(80.0, 250.0)):
    from oracle import oracle as O
    from flybrain import DeviceGraph, LIFCuda
    rng = np.random.default_rng(seed)
    idx = rng.choice(g.N, nd, replace=False)
    hz = rng.uniform(*rate, nd)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=seed)
    gb = LIFCuda(DeviceGraph(g), p, seed=seed)
    for i, h in zip(idx.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
        gb.setDriveOne(i, h)
    return ob, gb


def test_graph_has_repeats():
    g = repeated_graph()
    rows = [g.indices[g.indptr[r]:g.indptr[r + 1]] for r in range(g.N)]
    assert sum(len(r) != len(set(r.tolist())) for r in rows) > 100


@pytest.mark.parametrize("runner", ["stepwise", "multistep", "lagged"])
@pytest.mark.parametrize("variant", ["cuba", "coba_dep_bg"])
def test_repeated_targets_match_the_oracle(runner, variant):
    from flybrain import SYNTH_PARAMS
    from oracle import oracle as O
    from flybrain import _native as nat
    g = repeated_graph()
    p = dict(SYNTH_PARAMS) if variant == "cuba" else dict(SYNTH_PARAMS, coba=True, depU=0.1, bgRate=30.0, bgAmp=1.0)
    ob, gb = _pair(g, p, 7)
    steps = 300
    c0, r0 = ob.run(steps, raster=True)
    if runner == "stepwise":
        gb._batch.set_schedule(nat.FB_SCHEDULE_GRID)
        c1, r1 = gpu_stepwise(gb, steps)
    elif runner == "multistep":
        gb._batch.set_schedule(nat.FB_SCHEDULE_GRID)
        c1, r1 = gpu_multistep(gb, steps)
    else:
        c1, r1 = lagged_chunks(60)(gb, steps)
    np.testing.assert_array_equal(c1, c0)
    np.testing.assert_array_equal(r1, r0)
    assert_same_as_oracle(gb, ob, (runner, variant))
    assert int(c0.sum()) > 0


def test_repeated_targets_long_lagged_launch():
    """Unlogged 1,000-step launches of the delay-scheduled kernel, state and ring after each."""
    from flybrain import SYNTH_PARAMS
    from flybrain import _native as nat
    g = repeated_graph(N=6000, seed=23)
    ob, gb = _pair(g, dict(SYNTH_PARAMS, depU=0.05), 11, nd=120)
    gb._batch.set_schedule(nat.FB_SCHEDULE_LAGGED)
    for k in range(2):
        ob.run(1000)
        gb.run(1000)
        assert gb._batch.last_schedule() == nat.FB_SCHEDULE_LAGGED
        assert_same_as_oracle(gb, ob, k)


def test_more_than_four_repeats_is_refused():
    from flybrain import DeviceGraph
    from flybrain import _native as nat
    sign = np.ones(3, np.float32)
    ok = DeviceGraph(N=3, indptr=np.array([0, 4, 4, 4], np.uint32), indices=np.array([1, 2, 1, 1], np.uint32),
                     weights=np.ones(4, np.float32), sign=sign)
    assert ok.E == 4
    with pytest.raises(nat.FlyBrainError):
        DeviceGraph(N=3, indptr=np.array([0, 6, 6, 6], np.uint32), indices=np.array([1, 1, 1, 1, 1, 2], np.uint32),
                    weights=np.ones(6, np.float32), sign=sign)


def test_adjoint_with_repeated_targets_matches_the_oracle():
    """LIFDiff over a graph with repeated targets: the double-precision forward's tape and spike
    counts identical to the oracle's, every gradient within relative 1e-5."""
    from oracle.lifdiff_oracle import DiffProblem
    from flybrain.diff import DiffNet
    from test_adjoint_gpu import _compare_grads
    g = repeated_graph(N=1500, seed=31)
    params = dict(coba=True, soft=False, surrogateBeta=2.0, wSyn=0.5, minSyn=3.0, adaptInc=0.3, depU=0.1,
                  checkpoint=16)
    rng = np.random.default_rng(31)
    drv = rng.choice(g.N, 40, replace=False).astype(np.int32)
    hz = rng.uniform(50, 250, 40)
    prob = DiffProblem(g.N, g.indptr, g.indices, g.counts, g.sign, params=params, driven=drv, drive_hz=hz)
    net = DiffNet(dict(N=g.N, indptr=g.indptr, indices=g.indices, weights=g.counts, sign=g.sign), dict(params))
    for i, h in zip(drv.tolist(), hz.tolist()):
        net.setDriveOne(i, h)
    sc0, tape = prob.forward(150, seed=3, checkpoint=16)
    sc1 = net.forward(150, seed=3)
    assert sc0.tobytes() == sc1.tobytes()
    off, ix, amp = net.tape()
    np.testing.assert_array_equal(off, tape["off"])
    np.testing.assert_array_equal(ix, tape["idx"])
    dL = np.zeros(g.N, np.float32)
    dL[rng.choice(g.N, 200, replace=False)] = 1
    g0 = prob.backward(tape, dL)
    g1 = net.backward(dL)
    _compare_grads(g0, g1)
