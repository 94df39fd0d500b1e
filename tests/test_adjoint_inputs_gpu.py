"""LIFDiff's inputs beyond the network on the GPU (fb_diff_forward_ex): the drive schedule
(driveIdx/driveEpoch with setDriveOne order) and its gradient, driveSoft, a recorded spike train,
and the exact32 forward -- against the oracle, against the reference kernel's own golden run, and
against central differences of the GPU's forward.

Tolerances: hard-spike tapes are compared bit for bit; gradients in f64 mode within relative 1e-5
(the per-target inScale sums and a warp's gather are summed in another order than the oracle's);
the drive gradient is accumulated in float32 as the reference does, so relative 1e-4 there; finite
differences use the grad_check tolerance (scripts/grad_check.mjs:98)."""
import os

import numpy as np
import pytest

from adjoint_problem import P0, grad_check_inputs, within_tolerance
from test_adjoint_gpu import _close, _compare_grads

pytestmark = pytest.mark.gpu
LIF_KEYS = ("dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "wSyn", "adaptInc",
            "adaptTau", "depU", "depTau", "minSyn", "eExc", "eInh", "inhGain", "coba")


def _net(ins, params, driven=None, hz=None, driveIdx=None, extra=None):
    from flybrain.diff import DiffNet
    data = dict(N=ins["N"], indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"])
    opts = dict(params)
    for k in ("sizeLog", "thrMask", "biasMask", "logGain", "outScale", "thrOffset"):
        if ins.get(k) is not None:
            opts[k] = ins[k]
    if driveIdx is not None:
        opts["driveIdx"] = driveIdx
    opts.update(extra or {})
    net = DiffNet(data, opts)
    if driven is not None:
        for i, h in zip(driven, hz):
            net.setDriveOne(int(i), float(h))
    return net


def _pair(ins, params, driven=None, hz=None, driveIdx=None):
    from oracle.lifdiff_oracle import DiffProblem
    prob = DiffProblem(**ins, params=params, driven=driven, drive_hz=hz, driveIdx=driveIdx)
    return prob, _net(ins, params, driven, hz, driveIdx)


def _same_tape(net, tape):
    off, idx, amp = net.tape()
    np.testing.assert_array_equal(off, tape["off"])
    np.testing.assert_array_equal(idx, tape["idx"])
    np.testing.assert_array_equal(amp, tape["amp"])


def _twin():
    from conftest import GOLDEN
    from scenarios import load_case
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, "real_subgraph.npz"))
    z = np.load(os.path.join(GOLDEN, "adjoint", "real_subgraph_counts.npz"))
    EXC = np.array([0, 1, -1, -1, 1, 1, 1, -1], np.float32)
    (_, drv, hz), (_, bidx, bval), (_, steps) = meta["script"]
    bias_mask = np.zeros(int(z["N"]), np.uint8)
    bias_mask[bidx] = 1
    ins = dict(N=int(z["N"]), indptr=z["indptr"], indices=z["indices"], counts=z["counts"].astype(np.float32),
               sign=EXC[z["nt"]], biasMask=bias_mask)
    params = dict({k: meta["params"][k] for k in LIF_KEYS}, laminaBias=float(bval), exact32=True)
    return ins, params, np.array(drv, np.int32), np.array(hz), meta, blocks, steps


def test_exact32_forward_reproduces_the_reference_kernel_run():
    """exact32 on the GPU: the reference lif.c's own golden run (every step's fired list), and the
    oracle's exact32 tape and spike counts, bit for bit."""
    ins, params, drv, hz, meta, blocks, steps = _twin()
    prob, net = _pair(ins, params, drv, hz)
    sc1 = net.forward(steps, seed=meta["seed"])
    off, idx, _ = net.tape()
    counts0, raster0 = blocks[0]
    np.testing.assert_array_equal(np.diff(off), counts0)
    np.testing.assert_array_equal(idx, raster0)
    sc0, tape = prob.forward(steps, seed=meta["seed"])
    _same_tape(net, tape)
    assert sc0.tobytes() == sc1.tobytes()


def test_exact32_rejects_a_threshold_mask():
    from flybrain import _native as nat
    ins, params, drv, hz, meta, _, steps = _twin()
    ins["thrMask"] = np.zeros(ins["N"], np.uint8)
    ins["thrMask"][3] = 1
    net = _net(ins, params, drv, hz)
    with pytest.raises(nat.FlyBrainError, match="thr_mask"):
        net.forward(10)


def _schedule_case(seed=5):
    ins, params, drv, hz, meta, _, _ = _twin()
    params = dict(params, exact32=False, driveEpoch=25)
    rng = np.random.default_rng(seed)
    # driveIdx repeats a neuron (the last column naming it wins) and reaches beyond the driven set
    extra = [int(x) for x in rng.choice(ins["N"], 6, replace=False)]
    idx = np.array(list(drv[:12]) + extra + [int(drv[2])], np.int32)
    sched = rng.uniform(50, 300, (8, idx.shape[0])).astype(np.float32)
    sched[rng.random(sched.shape) < 0.3] = 0.0
    return ins, params, drv, hz, idx, sched


def test_drive_schedule_tape_is_identical_to_oracle():
    """Epoch-boundary setDriveOne edits of the drivenSet (removals keep order, re-insertions go to
    the end) reproduce the oracle's draw order: identical tapes and counts."""
    ins, params, drv, hz, idx, sched = _schedule_case()
    prob, net = _pair(ins, params, drv, hz, driveIdx=idx)
    steps = 25 * 8
    sc0, tape = prob.forward(steps, seed=3, driveAt=sched)
    sc1 = net.forward(steps, seed=3, driveAt=sched)
    _same_tape(net, tape)
    assert sc0.tobytes() == sc1.tobytes()
    assert tape["forced"].sum() > 50


def test_spike_train_tape_is_identical_to_oracle():
    ins, target = grad_check_inputs(seed=4)
    params = dict(P0, soft=False)
    rng = np.random.default_rng(4)
    driven = rng.choice(ins["N"], 20, replace=False).astype(np.int32)
    hz = rng.uniform(100, 300, 20)
    prob, net = _pair(ins, params, driven, hz)
    steps = 80
    train = [None] * steps
    for t in range(0, steps, 3):
        train[t] = [int(x) for x in rng.choice(ins["N"], 15)] + [int(driven[t % 20])]  # repeats included
    sc0, tape = prob.forward(steps, seed=2, spikeTrain=train)
    sc1 = net.forward(steps, seed=2, spikeTrain=train)
    _same_tape(net, tape)
    assert sc0.tobytes() == sc1.tobytes()


def _soft_drive_case():
    ins, target = grad_check_inputs(seed=8)
    rng = np.random.default_rng(8)
    didx = rng.choice(ins["N"], 12, replace=False).astype(np.int32)
    params = dict(P0, driveSoft=True, driveEpoch=10)
    sched = rng.uniform(40, 250, (6, 12)).astype(np.float32)
    return ins, target, didx, params, sched


def test_soft_drive_gradients_match_oracle():
    ins, target, didx, params, sched = _soft_drive_case()
    prob, net = _pair(ins, params, driveIdx=didx)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    sc0, tape = prob.forward(60, driveAt=sched)
    g0 = prob.backward(tape, dL)
    sc1 = net.forward(60, driveAt=sched)
    assert _close(sc0, sc1, rel=1e-6)
    g1 = net.backward(dL)
    _compare_grads(g0, g1)
    assert _close(g0["drive"], g1["drive"], rel=1e-4, abs_=1e-9)
    assert g1["clamped"]["drive"] == 0


@pytest.mark.parametrize("cell", [(0, 0), (2, 5), (5, 11)])
def test_drive_gradient_matches_gpu_finite_difference(cell):
    ins, target, didx, params, sched = _soft_drive_case()
    net = _net(ins, params, driveIdx=didx)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    L = float(net.forward(60, driveAt=sched)[target].astype(np.float64).sum())
    g = float(net.backward(dL)["drive"][cell])
    h = 2.0
    up, dn = sched.copy(), sched.copy()
    up[cell] += h
    dn[cell] -= h
    fd = (float(net.forward(60, record=False, driveAt=up)[target].astype(np.float64).sum())
          - float(net.forward(60, record=False, driveAt=dn)[target].astype(np.float64).sum())) / (2 * h)
    ok, rel = within_tolerance(g, fd, h, L)
    assert ok, (cell, g, fd, rel)


def test_hard_drive_gradient_through_forced_spikes_matches_oracle():
    """Hard spikes with a drawn drive: a forced spike's gradient reaches its epoch's drive value
    through ds/d(sd) = 1 (src/lifdiff.js:565-573); the scheduled drive also sets the draw odds."""
    ins, params, drv, hz, idx, sched = _schedule_case(seed=9)
    params = dict(params, surrogateBeta=2.0, adaptInc=0.2, checkpoint=16)
    prob, net = _pair(ins, params, drv, hz, driveIdx=idx)
    steps = 100
    sched = sched[:4]
    rng = np.random.default_rng(9)
    dL = rng.standard_normal(ins["N"]).astype(np.float32)
    _, tape = prob.forward(steps, seed=6, driveAt=sched)
    g0 = prob.backward(tape, dL)
    net.forward(steps, seed=6, driveAt=sched)
    _same_tape(net, tape)
    g1 = net.backward(dL)
    _compare_grads(g0, g1)
    assert _close(g0["drive"], g1["drive"], rel=1e-4, abs_=1e-7)
    assert np.abs(g1["drive"]).max() > 0


def test_drive_gradient_without_a_schedule_uses_the_drive_as_set():
    """driveIdx without driveAt: the drive as set, held every epoch (what the reference tapes when
    no onEpoch callback changes it), still yields a per-epoch drive gradient."""
    ins, target, didx, params, sched = _soft_drive_case()
    const = np.tile(np.linspace(60, 200, 12, dtype=np.float32), (6, 1))
    prob, _ = _pair(ins, params, driveIdx=didx)
    net = _net(ins, params, didx, const[0], driveIdx=didx)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    _, tape = prob.forward(60, driveAt=const)
    g0 = prob.backward(tape, dL)
    net.forward(60)
    g1 = net.backward(dL)
    assert _close(g0["drive"], g1["drive"], rel=1e-4, abs_=1e-9)


def test_batched_schedules_and_trains_match_single_networks():
    """fb_diff_batch_forward_ex: per-member schedules and spike trains, identical tapes and
    gradients to the members run alone."""
    from flybrain.diff import DiffBatch
    ins, params, drv, hz, idx, sched = _schedule_case(seed=11)
    params = dict(params, driveSoft=True, soft=True, driveEpoch=20)
    steps = 80
    scheds = [sched[:4], sched[4:8] * 0.5]
    rng = np.random.default_rng(11)
    trains = [None, [None if t % 4 else [int(x) for x in rng.choice(ins["N"], 8)] for t in range(steps)]]
    from flybrain.diff import DiffNet
    members = []
    for b in range(2):
        m = DiffNet(dict(N=ins["N"], indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"],
                         sign=ins["sign"]), dict(params, biasMask=ins["biasMask"], driveIdx=idx), _defer=True)
        for i, h in zip(drv, hz):
            m.setDriveOne(int(i), float(h))
        members.append(m)
    batch = DiffBatch(members, params)
    batch.forward([steps, steps], [3, 4], driveAt=scheds, spikeTrain=trains)
    dL = np.zeros(ins["N"], np.float32)
    dL[:50] = 1
    gb = batch.backward([dL, dL])
    for b in range(2):
        net = _net(ins, params, drv, hz, idx)
        net.forward(steps, seed=3 + b, driveAt=scheds[b], spikeTrain=trains[b])
        off, ix, amp = net.tape()
        off2, ix2, amp2 = batch.tape(b)
        np.testing.assert_array_equal(off, off2)
        np.testing.assert_array_equal(ix, ix2)
        np.testing.assert_array_equal(amp, amp2)
        g = net.backward(dL)
        for k, v in g["params"].items():
            assert v == gb[b]["params"][k], (b, k)
        np.testing.assert_array_equal(g["drive"], gb[b]["drive"])
