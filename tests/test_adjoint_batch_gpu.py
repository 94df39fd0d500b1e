"""Batches of differentiable brains (fb_diff_batch_*): every member's forward (spike counts,
tape) and backward (all gradients) are bit-identical to the same network run alone through
fb_diff_*, for members of different sizes, drives, seeds and lengths; the per-edge gradient
sum over members is the in-order double sum; arrays passed by the same object are shared."""
import numpy as np
import pytest

from adjoint_problem import P0, grad_check_inputs

pytestmark = pytest.mark.gpu

HARD = dict(coba=True, soft=False, surrogateBeta=2.0, wSyn=0.5, minSyn=3.0, adaptInc=0.3, depU=0.1,
            laminaBias=9.0, kcThreshold=2.0, inhGain=0.8, sizeAlpha=0.5, checkpoint=16)


def _members(params, rng_seed=0):
    from flybrain.diff import DiffNet
    from flybrain.synth import synth_graph
    out = []
    for s in (7, 8):
        ins, _ = grad_check_inputs(seed=s)
        data = dict(N=ins["N"], indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"])
        opts = dict(params, sizeLog=ins["sizeLog"], thrMask=ins["thrMask"], biasMask=ins["biasMask"],
                    logGain=np.zeros(ins["N"], np.float32), outScale=ins["outScale"], thrOffset=ins["thrOffset"])
        out.append((data, opts))
    g = synth_graph(900, 5)
    out.append((dict(N=g.N, indptr=g.indptr, indices=g.indices, weights=g.counts.astype(np.float32), sign=g.sign),
                dict(params)))
    rng = np.random.default_rng(rng_seed)
    nets = []
    for data, opts in out:
        drv = rng.choice(data["N"], 30, replace=False)
        hz = rng.uniform(80, 250, 30)
        pair = []
        for defer in (True, False):
            n = DiffNet(data, opts, _defer=defer)
            for i, h in zip(drv, hz):
                n.setDriveOne(int(i), float(h))
            if not defer:
                n._create(0)
            pair.append(n)
        nets.append(pair)
    return nets


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("mode", ["hard", "soft", "hard_f32"])
def test_batch_members_match_single_runs(mode):
    from flybrain.diff import DiffBatch
    params = dict(P0) if mode == "soft" else dict(HARD)
    if mode == "hard_f32":
        params["precision"] = "f32"
    pairs = _members(params)
    batch = DiffBatch([p[0] for p in pairs], params)
    steps, seeds = [90, 130, 70], [3, 4, 5]
    sc = batch.forward(steps, seeds)
    rng = np.random.default_rng(1)
    readouts = [np.sort(rng.choice(p[1].N, 40, replace=False)).astype(np.int32) for p in pairs]
    dls = [rng.normal(0, 1, (steps[b], 40)).astype(np.float32) for b in range(3)]
    gb = batch.backward(dls, readouts, truncate=50, lossFrom=10)
    for b, (_, single) in enumerate(pairs):
        sc1 = single.forward(steps[b], seed=seeds[b])
        _same(sc[b], sc1)
        for x, y in zip(batch.tape(b), single.tape()):
            _same(x, y)
        _same(batch.raster(b, readouts[b]), single.raster(readouts[b]))
        g1 = single.backward(dls[b], truncate=50, lossFrom=10, readout=readouts[b])
        assert gb[b]["params"] == g1["params"], (b, gb[b]["params"], g1["params"])
        assert gb[b]["clamped"] == g1["clamped"]
        for k in ("logGain", "edge", "bias", "outScale"):
            _same(gb[b][k], g1[k])
    assert any(np.abs(g["edge"]).sum() > 0 for g in gb)


def test_edge_sum_and_shared_arrays():
    from flybrain.diff import DiffBatch, DiffNet
    ins, _ = grad_check_inputs(seed=9)
    data = dict(N=ins["N"], indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"])
    eg = np.ones(ins["indices"].shape[0], np.float32)
    members = []
    rng = np.random.default_rng(2)
    for s in range(4):
        n = DiffNet(data, dict(HARD, edgeGain=eg), _defer=True)
        for i in rng.choice(ins["N"], 25, replace=False):
            n.setDriveOne(int(i), 150.0)
        members.append(n)
    batch = DiffBatch(members, HARD)
    batch.forward(100, seeds=[1, 2, 3, 4])
    dl = np.zeros(ins["N"], np.float32)
    dl[:100] = 1
    gs = batch.backward([dl] * 4)
    acc = gs[0]["edge"].copy()
    for g in gs[1:]:
        acc += g["edge"]
    _same(batch.edge_sum(), acc)
    _same(batch.edge_sum([2, 0]), gs[2]["edge"] + gs[0]["edge"])
    # the edge gains are one shared array: setting member 0's sets all four
    before = batch.forward(100, seeds=[1, 2, 3, 4])
    batch.set_array(0, "edgeGain", np.full(eg.shape[0], 1.5, np.float32))
    after = batch.forward(100, seeds=[1, 2, 3, 4])
    for b in range(4):
        assert after[b].sum() > before[b].sum()


def test_batch_rejects_bad_members():
    from flybrain._native import FlyBrainError
    from flybrain.diff import DiffBatch, DiffNet
    ins, _ = grad_check_inputs(seed=9)
    bad = np.array(ins["indices"], np.uint32)
    bad[5] = ins["N"]  # out of range
    n = DiffNet(dict(N=ins["N"], indptr=ins["indptr"], indices=bad, weights=ins["counts"], sign=ins["sign"]),
                HARD, _defer=True)
    with pytest.raises(FlyBrainError):
        DiffBatch([n], HARD)


def test_batched_rasters_equal_member_rasters():
    """fb_diff_batch_rasters (every member's readout raster in one call, into device buffers)
    gives each member's fb_diff_batch_raster, bit for bit, readouts of different sizes included."""
    import torch
    from flybrain.diff import DiffBatch
    pairs = _members(dict(HARD))
    batch = DiffBatch([p[0] for p in pairs], dict(HARD))
    steps = [90, 130, 70]
    batch.forward(steps, [3, 4, 5])
    rng = np.random.default_rng(2)
    readouts = [np.sort(rng.choice(p[1].N, n, replace=False)).astype(np.int32) for p, n in zip(pairs, (40, 25, 60))]
    outs = [torch.full((steps[b], readouts[b].shape[0]), -1.0, device="cuda") for b in range(3)]
    batch.rasters(readouts, outs)
    for b in range(3):
        _same(outs[b].cpu().numpy(), batch.raster(b, readouts[b]))
    assert sum(float(o.sum()) for o in outs) > 0


def test_captured_passes_equal_step_launches():
    """A forward and a backward replayed from captured CUDA graphs give what the same passes
    launched step by step give, bit for bit: at the capture, at a replay of the same key, after
    an input changed between replays (the graph reads it from device memory), and after more
    keys than the batch keeps (the first is evicted and captured again)."""
    from flybrain.diff import DiffBatch
    pairs = _members(dict(HARD))
    batch = DiffBatch([p[0] for p in pairs], dict(HARD))
    rng = np.random.default_rng(4)
    readouts = [np.sort(rng.choice(p[1].N, 40, replace=False)).astype(np.int32) for p in pairs]

    def run(steps, launches):
        batch.set_tuning(step_launches=launches)
        sc = batch.forward(steps, [3, 4, 5])
        tapes = [batch.tape(b) for b in range(3)]
        dls = [np.random.default_rng(steps[b]).normal(0, 1, (steps[b], 40)).astype(np.float32) for b in range(3)]
        gs = batch.backward(dls, readouts, truncate=40, lossFrom=5)
        return sc, tapes, gs

    def same_run(x, y):
        for b in range(3):
            _same(x[0][b], y[0][b])
            for u, v in zip(x[1][b], y[1][b]):
                _same(u, v)
            assert x[2][b]["params"] == y[2][b]["params"]
            for k in ("logGain", "edge", "bias", "outScale"):
                _same(x[2][b][k], y[2][b][k])

    steps = [90, 130, 70]
    ref = run(steps, True)
    same_run(run(steps, False), ref)  # captured
    same_run(run(steps, False), ref)  # replayed
    assert sum(float(np.abs(g["edge"]).sum()) for g in ref[2]) > 0
    batch.set_array(0, "outScale", np.full(pairs[0][1].N, 1.6, np.float32))
    ref2 = run(steps, True)
    same_run(run(steps, False), ref2)
    assert any(a.sum() != b.sum() for a, b in zip(ref2[0], ref[0]))
    for k in range(5):  # five more keys
        other = [s + 7 * (k + 1) for s in steps]
        same_run(run(other, False), run(other, True))
    same_run(run(steps, False), ref2)
