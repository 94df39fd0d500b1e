"""GPU parity of the brain step: the sm_103a kernel through the C ABI against the reference's
golden outputs and the oracle port. Integer/index results (rasters) and f32 state are compared
bit for bit (the bar for this path is exact equality, tolerance 0)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from scenarios import final_state, load_case, oracle_runner, run_scenario

pytestmark = pytest.mark.gpu
CASES = sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def gpu_stepwise(brain, n):
    """One launch per step, the fired list read back after each (LIFWasm.step semantics)."""
    counts, raster = [], []
    for _ in range(n):
        f = brain.step()
        counts.append(len(f))
        raster.append(f)
    return np.array(counts, np.int32), (np.concatenate(raster) if raster else np.zeros(0, np.int32))


def gpu_multistep(brain, n):
    """All n steps in one persistent launch; the device log records every step's fired list."""
    b = brain._batch
    b.record(n, 1 << 22)
    brain.run(n)
    counts, raster = b.spike_log(0, n, 1 << 22)
    b.record(0, 0)
    return counts, raster


def make_gpu_brain(meta, g):
    from flybrain import DeviceGraph, LIFCuda
    dg = DeviceGraph(N=meta["N"], indptr=g["indptr"], indices=g["indices"], weights=g["W"], sign=g["sign"])
    return LIFCuda(dg, meta["params"], seed=meta["seed"])


def assert_same(blocks, got, state, st):
    assert len(blocks) == len(got)
    for k, ((c0, r0), (c1, r1)) in enumerate(zip(blocks, got)):
        if not np.array_equal(c0, c1):
            bad = int(np.argmax(c0 != c1))
            raise AssertionError(f"block {k}: first divergent step {bad}: {c0[bad]} vs {c1[bad]}")
        np.testing.assert_array_equal(r1, r0)
    for k, v in state.items():
        assert v.tobytes() == st[k].tobytes(), f"state {k} differs: max |d| = {np.abs(v.astype(np.float64) - st[k]).max()}"


@pytest.mark.parametrize("case", CASES)
def test_golden_stepwise(case):
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, case))
    brain = make_gpu_brain(meta, g)
    got = run_scenario(brain, meta["script"], gpu_stepwise)
    assert_same(blocks, got, state, final_state(brain))


@pytest.mark.parametrize("case", CASES)
def test_golden_multistep(case):
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, case))
    brain = make_gpu_brain(meta, g)
    got = run_scenario(brain, meta["script"], gpu_multistep)
    assert_same(blocks, got, state, final_state(brain))


def test_sequential_mode_matches_exact():
    """The sequential delivery (used for presynaptic inhibition) on a case without it."""
    from flybrain import _native
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, "cuba_synth.npz"))
    brain = make_gpu_brain(meta, g)
    brain._batch.set_mode(_native.FB_DELIVER_SEQUENTIAL)
    got = run_scenario(brain, meta["script"], gpu_multistep)
    assert_same(blocks, got, state, final_state(brain))


def test_fast_mode_rates():
    """Float-atomic delivery: not bit-exact, but total activity within 5% of the reference."""
    from flybrain import _native
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, "real_subgraph.npz"))
    brain = make_gpu_brain(meta, g)
    brain._batch.set_mode(_native.FB_DELIVER_FAST)
    got = run_scenario(brain, meta["script"], gpu_multistep)
    ref = sum(int(c.sum()) for c, _ in blocks)
    new = sum(int(c.sum()) for c, _ in got)
    assert abs(new - ref) <= 0.05 * ref, (new, ref)


def _oracle_and_gpu(g, params, seed, idx, hz, steps, gpu_runner=gpu_multistep):
    from oracle import oracle as O
    from flybrain import DeviceGraph, LIFCuda
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, params, seed=seed)
    script = [["drive", idx.tolist(), hz.tolist()], ["step", steps]]
    ref = run_scenario(ob, script, oracle_runner)
    gb = LIFCuda(DeviceGraph(g), params, seed=seed)
    got = run_scenario(gb, script, gpu_runner)
    return ref, final_state(ob), got, final_state(gb)


def test_small_workload_full_window():
    """N=20,000, 150 Hz into 1%, 1,000 ms at dt 0.1: the raster is identical from step 0."""
    from flybrain import SYNTH_PARAMS, workload
    g, idx, hz, steps = workload("small")
    ref, s0, got, s1 = _oracle_and_gpu(g, SYNTH_PARAMS, 1, idx, hz, steps)
    assert_same(ref, got, s0, s1)


@pytest.mark.slow
def test_full_scale_window():
    """N=165,122 (~11M edges): the first 3,000 steps (300 ms) bit-identical to the oracle."""
    from flybrain import SYNTH_PARAMS, workload
    g, idx, hz, _ = workload("full")
    ref, s0, got, s1 = _oracle_and_gpu(g, SYNTH_PARAMS, 1, idx, hz, 3000)
    assert_same(ref, got, s0, s1)


def test_batch_uneven_matches_independent_brains():
    """Four brains with their own graphs, seeds, drives and step counts in one launch."""
    from oracle import oracle as O
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    rng = np.random.default_rng(5)
    graphs = [synth_graph(int(n), 40 + k) for k, n in enumerate((3000, 1200, 3000, 700))]
    dgs = [DeviceGraph(g) for g in graphs]
    params = [dict(SYNTH_PARAMS), dict(SYNTH_PARAMS, coba=True), dict(SYNTH_PARAMS, adaptInc=1.0),
              dict(SYNTH_PARAMS, depU=0.2)]
    seeds = [3, 4, 5, 6]
    steps = np.array([900, 0, 1500, 400], np.int32)
    batch = BrainBatch(dgs, params, seeds)
    drives = []
    for b, g in enumerate(graphs):
        idx = rng.choice(g.N, 30, replace=False).astype(np.int32)
        hz = rng.uniform(50, 250, 30)
        drives.append((idx, hz))
        batch.set_drive(b, idx, hz)
    batch.record(int(steps.max()), 1 << 20)
    batch.step_uneven(steps)
    for b, g in enumerate(graphs):
        ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, params[b], seed=seeds[b])
        for i, h in zip(*drives[b]):
            ob.setDriveOne(int(i), float(h))
        c0, r0 = ob.run(int(steps[b]), raster=True)
        c1, r1 = batch.spike_log(b, int(steps[b]), 1 << 20)
        np.testing.assert_array_equal(c1, c0)
        np.testing.assert_array_equal(r1, r0)
        for k in ("v", "gE", "gI", "refr", "adapt", "res", "spikeCount"):
            assert getattr(ob, k).tobytes() == batch.read(k, b).tobytes(), (b, k)
        assert batch.scalars(b)["rng"] == ob.rng
        assert batch.scalars(b)["head"] == ob.head


def test_invalid_arguments_are_rejected():
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    from flybrain._native import FlyBrainError
    g = synth_graph(500, 1)
    dg = DeviceGraph(g)
    b = BrainBatch([dg], SYNTH_PARAMS, [1])
    with pytest.raises(FlyBrainError):
        b.set_drive(0, [500], [10.0])
    with pytest.raises(FlyBrainError):
        b.set_bias(1, [0], [1.0])
    bad = g.indices.copy()
    bad[3] = g.N
    with pytest.raises(FlyBrainError):
        DeviceGraph(N=g.N, indptr=g.indptr, indices=bad, weights=g.weights, sign=g.sign)
    with pytest.raises(FlyBrainError):  # one-step delay ring
        BrainBatch([dg], dict(SYNTH_PARAMS, delay=0.1), [1])
    # the handle still works after rejected calls
    b.set_drive(0, [1, 2], [100.0, 100.0])
    b.step(10)


def _six_brain_batch():
    """Six brains (more than the kernel caches headers for) of uneven sizes, each against the
    oracle, bit for bit."""
    from oracle import oracle as O
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    rng = np.random.default_rng(6)
    sizes = (2100, 900, 4000, 1500, 3100, 700)
    graphs = [synth_graph(n, 60 + k) for k, n in enumerate(sizes)]
    batch = BrainBatch([DeviceGraph(g) for g in graphs], SYNTH_PARAMS, list(range(1, 7)))
    steps = rng.integers(300, 900, len(sizes)).astype(np.int32)
    oracles = []
    for b, g in enumerate(graphs):
        idx = rng.choice(g.N, min(g.N // 4, 700), replace=False).astype(np.int32)
        hz = rng.uniform(50, 250, idx.shape[0])
        batch.set_drive(b, idx, hz)
        ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, SYNTH_PARAMS, seed=b + 1)
        for i, h in zip(idx, hz):
            ob.setDriveOne(int(i), float(h))
        oracles.append(ob)
    batch.record(int(steps.max()), 1 << 21)
    batch.step_uneven(steps)
    for b, ob in enumerate(oracles):
        c0, r0 = ob.run(int(steps[b]), raster=True)
        c1, r1 = batch.spike_log(b, int(steps[b]), 1 << 21)
        np.testing.assert_array_equal(c1, c0)
        np.testing.assert_array_equal(r1, r0)
        assert ob.v.tobytes() == batch.read("v", b).tobytes()


def test_batch_more_brains_than_cached_headers():
    _six_brain_batch()


def test_checked_build_finds_no_bad_index():
    """The same batch under the index-checked library (every data-dependent index bounds-checked
    on the device, failures reported by fb_step) in a fresh process."""
    import subprocess
    import sys
    from conftest import ROOT
    code = ("import sys; sys.path[:0] = [%r, %r, %r]; import test_step_gpu as t; t._six_brain_batch()"
            % (ROOT, os.path.join(ROOT, "fly-brain_gb300"), os.path.dirname(os.path.abspath(__file__))))
    env = dict(os.environ, FLYBRAIN_CHECKED="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr


def test_synchronous_burst_into_one_target():
    """~150 presynaptic spikes reach one neuron in the same step: more contributions than a
    target's in-place bucket and local sort hold, still summed in the reference's order."""
    from oracle import oracle as O
    from flybrain import DeviceGraph, LIFCuda, SYNTH_PARAMS
    N = 500
    rows = [[499, (p * 7) % 450 + 40] if p < 300 else [(p * 13) % 499] for p in range(N)]
    rows = [sorted(set(r)) for r in rows]
    indptr = np.zeros(N + 1, np.uint32)
    indptr[1:] = np.cumsum([len(r) for r in rows])
    indices = np.concatenate([np.array(r, np.uint32) for r in rows])
    rng = np.random.default_rng(3)
    W = rng.uniform(0.5, 3.0, indices.shape[0]).astype(np.float32)
    sign = np.where(rng.random(N) < 0.7, 1.0, -1.0).astype(np.float32)
    p = dict(SYNTH_PARAMS)
    ob = O.OracleBrain(N, indptr, indices, W, sign, p, seed=9)
    gb = LIFCuda(DeviceGraph(N=N, indptr=indptr, indices=indices, weights=W, sign=sign), p, seed=9)
    for i in range(300):
        ob.setDriveOne(i, 4000.0)
        gb.setDriveOne(i, 4000.0)
    c0, r0 = ob.run(400, raster=True)
    c1, r1 = gpu_multistep(gb, 400)
    np.testing.assert_array_equal(c1, c0)
    np.testing.assert_array_equal(r1, r0)
    assert c0.max() > 100
    for k in ("v", "gE", "gI"):
        assert getattr(ob, k).tobytes() == getattr(gb, k).tobytes(), k


def test_large_batches_created_in_either_order():
    """Two batches whose per-brain launch tables need more than 48 KB of shared memory, the
    larger created first: both still launch and step like a lone brain of the same seed."""
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    g = synth_graph(60, 3)
    dg = DeviceGraph(g)
    big = BrainBatch([dg] * 1300, SYNTH_PARAMS, list(range(1, 1301)))
    small = BrainBatch([dg] * 1150, SYNTH_PARAMS, list(range(1, 1151)))
    lone = BrainBatch([dg], SYNTH_PARAMS, [7])
    for batch in (big, small, lone):
        batch.set_drive(0 if batch is lone else 6, np.arange(0, 60, 3, dtype=np.int32), 400.0)
        batch.step(50)
    for batch in (big, small):
        assert batch.read("v", 6).tobytes() == lone.read("v", 0).tobytes()
        assert batch.read("spikeCount", 6).tobytes() == lone.read("spikeCount", 0).tobytes()


def test_set_params_between_steps_matches_the_oracle():
    """LIFGpu.setParams on the device brain (fb_set_params): the membrane and synaptic constants,
    adaptation, depression, background and COBA change between two runs; the oracle's header
    gets the same constants (LIFWasm._writeHeader); rasters and state agree bit for bit."""
    from oracle import oracle as O
    from flybrain import LIFCuda, SYNTH_PARAMS, synth_graph
    g = synth_graph(3000, 17)
    p = dict(SYNTH_PARAMS, wSyn=1.6)
    brain = LIFCuda(g, p, seed=4)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=4)
    rng = np.random.default_rng(17)
    for i in rng.choice(g.N, 60, replace=False):
        brain.setDriveOne(int(i), 220.0)
        ob.setDriveOne(int(i), 220.0)
    brain.setBias([1, 2, 3], 2.0)
    ob.setBias([1, 2, 3], 2.0)
    brain._batch.record(300, 1 << 20)
    c0a, r0a = ob.run(150, raster=True)
    brain.run(150)
    q = dict(tauM=15.0, vThresh=-46.0, tauSyn=4.0, adaptInc=0.5, depU=0.1, bgRate=20.0, bgAmp=0.8, coba=True)
    brain.setParams(q)
    ob.p.update(q)
    h = ob._pull()
    for k, v in enumerate(O.header_constants(ob.p)):
        h.c[k] = float(v)
    h.coba = 1
    h.bgEvents = float(np.float32(g.N * ob.p["bgRate"] * ob.p["dt"] / 1000))
    h.bgAmp = float(np.float32(ob.p["bgAmp"]))
    ob._push()
    c0b, r0b = ob.run(150, raster=True)
    brain.run(150)
    c1, r1 = brain._batch.spike_log(0, 300, 1 << 20)
    np.testing.assert_array_equal(c1, np.concatenate([c0a, c0b]))
    np.testing.assert_array_equal(r1, np.concatenate([r0a, r0b]))
    for k in ("v", "gE", "gI", "refr", "trace", "adapt", "res", "spikeCount"):
        assert getattr(brain, k).tobytes() == np.asarray(getattr(ob, k)).tobytes(), k
    with pytest.raises(Exception, match="ring"):
        brain.setParams(dict(delay=3.0))
