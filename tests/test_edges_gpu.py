"""Edge cases of every GPU path against the oracle: a graph with no edges, a single neuron, no
drive, every neuron driven, zero-step calls, both step schedules; LIFDiff and flyvis without
edges. Results compared bit for bit (integer rasters and f32 state, tolerance 0)."""
import numpy as np
import pytest

from scenarios import final_state, oracle_runner, run_scenario
from test_step_gpu import assert_same, gpu_multistep

pytestmark = pytest.mark.gpu


def _graph(N, E_per=0, seed=0, self_loop=False):
    """A small CSR graph: E_per distinct random targets per row (or one self-edge per neuron)."""
    from flybrain.synth import Graph
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(N):
        if self_loop:
            rows.append(np.array([i]))
        else:
            rows.append(np.sort(rng.choice(N, min(E_per, N), replace=False)) if E_per else np.zeros(0, np.int64))
    indptr = np.zeros(N + 1, np.uint32)
    indptr[1:] = np.cumsum([r.shape[0] for r in rows])
    indices = np.concatenate(rows).astype(np.uint32) if indptr[-1] else np.zeros(0, np.uint32)
    w = rng.uniform(0.5, 3.0, indices.shape[0]).astype(np.float32)
    sign = np.where(rng.random(N) < 0.7, 1.0, -1.0).astype(np.float32)
    return Graph(N, indptr, indices, w, sign)


def _both_schedules(g, params, script, seed=3):
    from oracle import oracle as O
    from flybrain import DeviceGraph, LIFCuda
    from flybrain import _native as nat
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, params, seed=seed)
    ref = run_scenario(ob, script, oracle_runner)
    s0 = final_state(ob)
    for sched in (nat.FB_SCHEDULE_GRID, nat.FB_SCHEDULE_LAGGED):
        gb = LIFCuda(DeviceGraph(g), params, seed=seed)
        gb._batch.set_schedule(sched)
        got = run_scenario(gb, script, gpu_multistep if sched == nat.FB_SCHEDULE_GRID else _lagged_runner)
        assert_same(ref, got, s0, final_state(gb))


def _lagged_runner(brain, n):
    """Launches of at most 64 steps (the per-step log of the delay-scheduled kernel)."""
    counts, raster = [], []
    left = n
    while left > 0:
        c = min(64, left)
        k, r = gpu_multistep(brain, c)
        counts.append(k)
        raster.append(r)
        left -= c
    if not counts:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    return np.concatenate(counts), np.concatenate(raster)


def test_no_edges():
    from flybrain import SYNTH_PARAMS
    g = _graph(200, 0)
    assert g.E == 0
    _both_schedules(g, dict(SYNTH_PARAMS), [["drive", list(range(0, 200, 7)), [300.0] * 29], ["bias", [1, 2], 9.0],
                                            ["step", 300]])


def test_single_neuron():
    from flybrain import SYNTH_PARAMS
    g = _graph(1, self_loop=True)
    _both_schedules(g, dict(SYNTH_PARAMS, wSyn=4.0), [["drive", [0], [250.0]], ["step", 400]])


def test_no_drive_stays_at_rest():
    from flybrain import SYNTH_PARAMS
    g = _graph(500, 20, seed=2)
    _both_schedules(g, dict(SYNTH_PARAMS), [["step", 200]])


def test_every_neuron_driven():
    from flybrain import SYNTH_PARAMS
    g = _graph(300, 15, seed=4)
    _both_schedules(g, dict(SYNTH_PARAMS, coba=True), [["drive", list(range(300)), [120.0] * 300], ["step", 300]])


def test_zero_steps_change_nothing():
    from flybrain import DeviceGraph, LIFCuda, SYNTH_PARAMS
    g = _graph(100, 10, seed=5)
    gb = LIFCuda(DeviceGraph(g), dict(SYNTH_PARAMS), seed=1)
    gb.setDriveOne(3, 500.0)
    gb.run(25)
    before = final_state(gb)
    gb.run(0)
    gb._batch.step_uneven(np.zeros(1, np.int32))
    after = final_state(gb)
    for k, v in before.items():
        assert v.tobytes() == after[k].tobytes(), k


def test_diff_without_edges_or_drive():
    """LIFDiff on a graph with no edges: the oracle's forward and gradients, all finite."""
    from adjoint_problem import P0
    from oracle.lifdiff_oracle import DiffProblem
    from flybrain.diff import DiffNet
    N = 64
    ins = dict(N=N, indptr=np.zeros(N + 1, np.uint32), indices=np.zeros(0, np.uint32),
               counts=np.zeros(0, np.float32), sign=np.ones(N, np.float32))
    prob = DiffProblem(**ins, params=P0)
    net = DiffNet(dict(N=N, indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"]),
                  dict(P0))
    dL = np.ones(N, np.float32)
    sc0, tape = prob.forward(40)
    g0 = prob.backward(tape, dL)
    sc1 = net.forward(40)
    g1 = net.backward(dL)
    assert sc0.tobytes() == sc1.tobytes()
    for k, v in g0["params"].items():
        assert np.isfinite(g1["params"][k]) and np.isclose(v, g1["params"][k], rtol=1e-6, atol=1e-12), k
    assert g1["edge"].shape == (0,)


def test_flyvis_without_edges():
    from oracle import oracle as O
    from flybrain.flyvis import FlyVis
    N = 100
    rng = np.random.default_rng(1)
    m = dict(N=N, E=0, indptr=np.zeros(N + 1, np.int32), target=np.zeros(0, np.int32), weight=np.zeros(0, np.float32),
             bias=rng.normal(0, 1, N).astype(np.float32), tau=rng.uniform(0.02, 0.2, N).astype(np.float32), dt=0.02)
    x = rng.normal(0, 1, (2, N)).astype(np.float32)
    fv = FlyVis(m, B=2)
    for b in range(2):
        fv.write("x", b, x[b])
    fv.step(10)
    v = np.tile(m["bias"], (2, 1)).astype(np.float32)
    O.fv_run(m, v, x, 10)
    for b in range(2):
        assert fv.v(b).tobytes() == v[b].tobytes()


def test_signed_zero_and_restored_parameters():
    """bias and thr written as -0.0, as nonzero values and back to +0.0: each write leaves the
    step's arithmetic that of lif.c (the update stops treating the field as all +0.0 once a word
    other than +0.0 is stored)."""
    from flybrain import SYNTH_PARAMS
    g = _graph(400, 12, seed=9)
    N = g.N
    every = list(range(N))
    script = [["drive", list(range(0, N, 5)), [220.0] * len(range(0, N, 5))],
              ["bias", every, -0.0], ["thr", [3], [-0.0]], ["step", 120],
              ["bias", list(range(0, N, 3)), 2.5], ["thr", list(range(1, N, 4)), [-1.5] * len(range(1, N, 4))],
              ["step", 120], ["bias", every, 0.0], ["thr", every, [0.0] * N], ["step", 120]]
    _both_schedules(g, dict(SYNTH_PARAMS), script)
