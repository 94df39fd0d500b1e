"""The autotuner's knobs on the GPU: every launch shape gives the oracle's rasters bit for bit
(grid schedule: resident CTAs per SM x edges per warp item) and identical gradients (adjoint:
K, per-neuron and per-arrival blocks); the tuner itself searches and applies a valid shape."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch():
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    rng = np.random.default_rng(21)
    graphs = [synth_graph(int(n), 70 + k) for k, n in enumerate((3000, 1500, 2500))]
    batch = BrainBatch([DeviceGraph(g) for g in graphs], dict(SYNTH_PARAMS, wSyn=1.6), [7, 8, 9])
    drives = []
    for b, g in enumerate(graphs):
        idx = rng.choice(g.N, 60, replace=False).astype(np.int32)
        hz = rng.uniform(100, 300, 60)
        drives.append((idx, hz))
        batch.set_drive(b, idx, hz)
    return batch, graphs, drives


@pytest.mark.parametrize("shape", [(1, 1), (1, 64), (0, 3), (0, 16)])
def test_grid_launch_shape_keeps_the_oracle_raster(shape):
    from oracle import oracle as O
    from flybrain import SYNTH_PARAMS
    from flybrain import _native as nat
    batch, graphs, drives = _batch()
    t = batch.tuning()
    bps = shape[0] or t["max_blocks_per_sm"]
    batch.set_tuning(bps, shape[1])
    assert batch.tuning()["blocks_per_sm"] == bps and batch.tuning()["item_chunks"] == shape[1]
    batch.set_schedule(nat.FB_SCHEDULE_GRID)
    steps = 600
    batch.record(steps, 1 << 20)
    batch.step(steps)
    for b, g in enumerate(graphs):
        ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, dict(SYNTH_PARAMS, wSyn=1.6), seed=7 + b)
        for i, h in zip(*drives[b]):
            ob.setDriveOne(int(i), float(h))
        c0, r0 = ob.run(steps, raster=True)
        c1, r1 = batch.spike_log(b, steps, 1 << 20)
        np.testing.assert_array_equal(c1, c0)
        np.testing.assert_array_equal(r1, r0)
        assert ob.v.tobytes() == batch.read("v", b).tobytes()


def test_dynamic_sub_tile_dealing_keeps_the_rasters():
    """160 brains, enough sub-tiles per warp for the update phase to hand the last 3/8 out from a
    counter: every brain's raster and state equal the all-dealt launch's, and two brains the
    oracle's."""
    from oracle import oracle as O
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    from flybrain import _native as nat
    g = synth_graph(12000, 91)
    B, steps = 160, 200
    rng = np.random.default_rng(5)
    drives = [(np.sort(rng.choice(g.N, 150, replace=False)).astype(np.int32), rng.uniform(80, 300, 150))
              for _ in range(B)]
    p = dict(SYNTH_PARAMS, wSyn=1.6)
    out = []
    for grab in (-1, 3):
        topo = DeviceGraph(g)
        batch = BrainBatch([topo] * B, p, list(range(11, 11 + B)))
        for b, (idx, hz) in enumerate(drives):
            batch.set_drive(b, idx, hz)
        batch.set_tuning(1, 2, grab)
        assert batch.tuning()["sub_grab"] == grab
        batch.set_schedule(nat.FB_SCHEDULE_GRID)
        batch.record(steps, 1 << 18)
        batch.step(steps)
        out.append([(batch.spike_log(b, steps, 1 << 18), batch.read("v", b)) for b in range(B)])
    for b in range(B):
        (c0, r0), v0 = out[0][b]
        (c1, r1), v1 = out[1][b]
        np.testing.assert_array_equal(c0, c1)
        np.testing.assert_array_equal(r0, r1)
        assert v0.tobytes() == v1.tobytes()
    for b in (0, B - 1):
        ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=11 + b)
        for i, h in zip(*drives[b]):
            ob.setDriveOne(int(i), float(h))
        c, r = ob.run(steps, raster=True)
        (c1, r1), v1 = out[1][b]
        np.testing.assert_array_equal(c1, c)
        np.testing.assert_array_equal(r1, r)
        assert ob.v.tobytes() == v1.tobytes()


def test_uneven_batch_with_dynamic_dealing_keeps_the_rasters():
    """160 brains stepped unevenly (60-200 steps) in one launch: as brains finish, the update's
    sub-tiles are renumbered over the ones still stepping and the counter-dealt tail switches off;
    every brain's raster and state equal those of the all-dealt launch, two brains the oracle's."""
    from oracle import oracle as O
    from flybrain import BrainBatch, DeviceGraph, SYNTH_PARAMS, synth_graph
    from flybrain import _native as nat
    g = synth_graph(12000, 93)
    B = 160
    rng = np.random.default_rng(6)
    steps = rng.integers(60, 201, B).astype(np.int32)
    drives = [(np.sort(rng.choice(g.N, 150, replace=False)).astype(np.int32), rng.uniform(80, 300, 150))
              for _ in range(B)]
    p = dict(SYNTH_PARAMS, wSyn=1.6)
    out = []
    for grab in (-1, 4):
        batch = BrainBatch([DeviceGraph(g)] * B, p, list(range(21, 21 + B)))
        for b, (idx, hz) in enumerate(drives):
            batch.set_drive(b, idx, hz)
        batch.set_tuning(1, 2, grab)
        batch.set_schedule(nat.FB_SCHEDULE_GRID)
        batch.record(200, 1 << 18)
        batch.step_uneven(steps)
        out.append([(batch.spike_log(b, int(steps[b]), 1 << 18), batch.read("v", b)) for b in range(B)])
    for b in range(B):
        (c0, r0), v0 = out[0][b]
        (c1, r1), v1 = out[1][b]
        np.testing.assert_array_equal(c0, c1)
        np.testing.assert_array_equal(r0, r1)
        assert v0.tobytes() == v1.tobytes()
    for b in (int(np.argmin(steps)), int(np.argmax(steps))):
        ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=21 + b)
        for i, h in zip(*drives[b]):
            ob.setDriveOne(int(i), float(h))
        c, r = ob.run(int(steps[b]), raster=True)
        (c1, r1), v1 = out[1][b]
        np.testing.assert_array_equal(c1, c)
        np.testing.assert_array_equal(r1, r)
        assert ob.v.tobytes() == v1.tobytes()


def test_tuning_is_validated():
    from flybrain import _native as nat
    batch, _, _ = _batch()
    t = batch.tuning()
    with pytest.raises(nat.FlyBrainError):
        batch.set_tuning(t["max_blocks_per_sm"] + 1, 1)
    with pytest.raises(nat.FlyBrainError):
        batch.set_tuning(1, 65)
    with pytest.raises(nat.FlyBrainError):
        batch.set_tuning(1, 1, 257)
    with pytest.raises(nat.FlyBrainError):
        batch.set_tuning(1, 1, -2)


def test_tune_brains_applies_a_valid_shape(tmp_path, monkeypatch):
    from flybrain.autotune import tune_brains
    monkeypatch.setenv("FLYBRAIN_TUNE_CACHE", str(tmp_path / "tune.json"))
    batch, _, _ = _batch()
    r = tune_brains(batch, steps=50, item_chunks=(1, 4), repeats=1)
    t = batch.tuning()
    assert (t["blocks_per_sm"], t["item_chunks"]) == (r["blocks_per_sm"], r["item_chunks"])
    assert len(r["table"]) == 2 * t["max_blocks_per_sm"] and not r["cached"]
    assert tune_brains(batch, steps=50)["cached"]


def _diff_batch():
    from adjoint_problem import P0, grad_check_inputs
    from flybrain.diff import DiffBatch, DiffNet
    ins, target = grad_check_inputs(seed=3)
    data = dict(N=ins["N"], indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"])
    rng = np.random.default_rng(3)
    members = []
    for b in range(3):
        m = DiffNet(data, dict(P0, sizeLog=ins["sizeLog"], thrMask=ins["thrMask"], biasMask=ins["biasMask"]),
                    _defer=True)
        for i in rng.choice(ins["N"], 30, replace=False):
            m.setDriveOne(int(i), float(rng.uniform(50, 250)))
        members.append(m)
    batch = DiffBatch(members, dict(P0, soft=False, surrogateBeta=2.0))
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    return batch, [dL] * 3


def test_adjoint_launch_shape_and_checkpoint_keep_the_gradients():
    batch, dLs = _diff_batch()
    steps, seeds = [120, 90, 120], [1, 2, 3]
    batch.forward(steps, seeds, checkpoint=16)
    tapes = [batch.tape(b) for b in range(3)]
    g0 = batch.backward(dLs)
    for nb, ab, K in ((1, 2, 16), (3, 64, 16), (2, 5, 40)):
        batch.set_tuning(nb, ab)
        batch.forward(steps, seeds, checkpoint=K)
        for b in range(3):
            for x, y in zip(tapes[b], batch.tape(b)):
                np.testing.assert_array_equal(x, y)
        g1 = batch.backward(dLs)
        # a replay reproduces the forward bit for bit from any checkpoint, and the reverse sweep
        # visits steps in the same order, so K changes nothing either
        for b in range(3):
            for k, v in g0[b]["params"].items():
                assert v == g1[b]["params"][k], (nb, ab, K, b, k)
            np.testing.assert_array_equal(g0[b]["edge"], g1[b]["edge"])
            np.testing.assert_array_equal(g0[b]["logGain"], g1[b]["logGain"])


def test_tune_diff_applies_a_valid_shape(tmp_path, monkeypatch):
    from flybrain.autotune import tune_diff
    monkeypatch.setenv("FLYBRAIN_TUNE_CACHE", str(tmp_path / "tune.json"))
    batch, dLs = _diff_batch()
    r = tune_diff(batch, [100] * 3, [1, 2, 3], dLs, Ks=(16, 50), neuron_blocks=(1, 2), arrival_blocks=(2, 8))
    assert r["checkpoint"] in (16, 50, batch.members[0].p["checkpoint"]) and batch.p["checkpoint"] == r["checkpoint"]
    assert batch.tuning == dict(neuron_blocks=r["neuron_blocks"], arrival_blocks=r["arrival_blocks"],
                                step_launches=False)  # timed with step launches, then restored
    assert len(r["table"]) == 1 + 1 + 1 + 2 + 2  # warm-up, K0 = 16, K = 50, two of each grid knob
