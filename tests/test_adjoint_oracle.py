"""The adjoint oracle (a C restatement of LIFDiff) against central finite differences of its own
smooth forward pass: the check scripts/grad_check.mjs runs, on the same kind of problem."""
import numpy as np
import pytest

from adjoint_problem import H, P0, grad_check_inputs, within_tolerance
from oracle.lifdiff_oracle import DIFF_PARAMS, DiffProblem

STEPS = 60


@pytest.fixture(scope="module")
def problem():
    ins, target = grad_check_inputs()
    prob = DiffProblem(**ins, params=P0)
    dL = np.zeros(prob.N, np.float32)
    dL[target] = 1
    sc, tape = prob.forward(STEPS)
    g = prob.backward(tape, dL)
    return prob, target, float(sc[target].astype(np.float64).sum()), g


def loss(prob, target, **over):
    sc, _ = prob.forward(STEPS, **over)
    return float(sc[target].astype(np.float64).sum())


@pytest.mark.parametrize("name", DIFF_PARAMS)
def test_global_gradient_matches_finite_difference(problem, name):
    prob, target, L, g = problem
    h = H[name]
    fd = (loss(prob, target, **{name: P0[name] + h}) - loss(prob, target, **{name: P0[name] - h})) / (2 * h)
    ok, rel = within_tolerance(g["params"][name], fd, h, L)
    assert ok, (name, g["params"][name], fd, rel)


@pytest.mark.parametrize("i", [0, 1, 2, 200, 300])
def test_log_gain_gradient_matches_finite_difference(problem, i):
    prob, target, L, g = problem
    h = 2e-2
    up, dn = prob.logGain.copy(), prob.logGain.copy()
    up[i] += h
    dn[i] -= h
    fd = (loss(prob, target, logGainArr=up) - loss(prob, target, logGainArr=dn)) / (2 * h)
    ok, rel = within_tolerance(float(g["logGain"][i]), fd, h, L)
    assert ok, (i, float(g["logGain"][i]), fd, rel)


def test_edge_and_bias_gradients_are_consistent(problem):
    """The per-edge and per-neuron extras agree with the reference's own outputs they refine:
    sum_j gEdge_j * dW_j/dwSyn reproduces the wSyn gradient's delivery part, and the per-neuron
    bias gradient summed over the laminaBias neurons is the laminaBias gradient."""
    prob, target, L, g = problem
    lam = float(g["gBias"][prob.biasMask.astype(bool)].sum())
    assert abs(lam - g["params"]["laminaBias"]) <= 1e-6 * max(1.0, abs(lam))
    assert np.isfinite(g["gEdge"]).all() and np.abs(g["gEdge"]).sum() > 0


# ---- the drive as an input, recorded spike trains, and the exact32 twin -----------------------

LIF_KEYS = ("dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "wSyn", "adaptInc",
            "adaptTau", "depU", "depTau", "minSyn", "eExc", "eInh", "inhGain", "coba")


def _twin_case():
    """The golden real-connectome case (tests/golden/real_subgraph.npz, made by the reference lif.c)
    and the same 600-neuron subgraph's raw counts (tests/golden/adjoint/)."""
    import json
    import os
    from conftest import GOLDEN
    from scenarios import load_case
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, "real_subgraph.npz"))
    z = np.load(os.path.join(GOLDEN, "adjoint", "real_subgraph_counts.npz"))
    EXC = np.array([0, 1, -1, -1, 1, 1, 1, -1], np.float32)
    prm = {k: meta["params"][k] for k in LIF_KEYS}
    (_, drv, hz), (_, bidx, bval), (_, steps) = meta["script"]
    bias_mask = np.zeros(int(z["N"]), np.uint8)
    bias_mask[bidx] = 1
    prob = DiffProblem(int(z["N"]), z["indptr"], z["indices"], z["counts"].astype(np.float32), EXC[z["nt"]],
                       params=dict(prm, laminaBias=float(bval), exact32=True), biasMask=bias_mask,
                       driven=np.array(drv, np.int32), drive_hz=np.array(hz))
    return prob, meta, blocks, state, steps


def test_exact32_forward_is_the_reference_kernel():
    """exact32 (src/lifdiff.js:105-109) makes LIFDiff's hard forward bit-identical to lif.c: every
    step's fired list of the reference's own golden run, and the final state, reproduced."""
    prob, meta, blocks, state, steps = _twin_case()
    sc, tape = prob.forward(steps + 1, seed=meta["seed"], checkpoint=steps)
    counts0, raster0 = blocks[0]
    counts = np.diff(tape["off"])[:steps]
    np.testing.assert_array_equal(counts, counts0)
    np.testing.assert_array_equal(tape["idx"][: tape["off"][steps]], raster0)
    N = prob.N
    ck = tape["ckpt"][N * 6: N * 12]  # the state after `steps` steps
    for a, name in enumerate(("v", "gE", "gI", "adapt", "res", "refr")):
        assert ck[a * N:(a + 1) * N].tobytes() == state[name].tobytes(), name


def test_drive_schedule_follows_setDriveOne_order():
    """driveAt sets driveIdx's rates at epoch boundaries with setDriveOne semantics: a neuron set
    to zero leaves the draw order and rejoins at its end. Against lif.c's stream (OracleBrain, the
    LIFWasm restatement) driven through the same setDriveOne calls."""
    from oracle import oracle as O
    prob, meta, blocks, state, steps = _twin_case()
    drv = list(meta["script"][0][1])
    rng = np.random.default_rng(5)
    idx = np.array(drv[:12] + [int(x) for x in rng.choice(prob.N, 6, replace=False)], np.int32)
    ep, n_ep = 25, 8
    sched = rng.uniform(50, 300, (n_ep, idx.shape[0])).astype(np.float32)
    sched[rng.random(sched.shape) < 0.3] = 0.0
    prob.driveIdx = idx
    _, tape = prob.forward(ep * n_ep, seed=3, driveEpoch=ep, driveAt=sched)
    # lif.c through the restated LIFWasm glue, compiled W as writeGraph makes it
    p = dict(meta["params"])
    W, sign = O.write_graph_f64(prob.N, prob.indptr, prob.indices, prob.counts, prob.sign, p)
    ob = O.OracleBrain(prob.N, prob.indptr, prob.indices, W, sign, p, seed=3)
    for i, h in zip(drv, meta["script"][0][2]):
        ob.setDriveOne(int(i), float(h))
    ob.setBias(list(meta["script"][1][1]), float(meta["script"][1][2]))
    ref = []
    for e in range(n_ep):
        for k, i in enumerate(idx):
            ob.setDriveOne(int(i), float(sched[e, k]))
        c, r = ob.run(ep, raster=True)
        ref.append((c, r))
    counts = np.concatenate([c for c, _ in ref])
    raster = np.concatenate([r for _, r in ref])
    np.testing.assert_array_equal(np.diff(tape["off"]), counts)
    np.testing.assert_array_equal(tape["idx"], raster)


def test_spike_train_forces_recorded_spikes():
    """spikeTrain[t] forces its neurons at step t (after the drive, skipping refractory ones),
    with no draw; they lead the step's list as forced spikes (src/lifdiff.js:298-306)."""
    ins, _ = grad_check_inputs(seed=4)
    prob = DiffProblem(**ins, params=dict(P0, soft=False, tRef=2.2))
    steps = 40
    train = [[] for _ in range(steps)]
    train[3] = [5, 17, 5]          # a repeat is refractory the second time
    train[5] = [17, 30]            # 17 is still refractory from step 3
    _, tape = prob.forward(steps, seed=2, spikeTrain=train)
    f3 = tape["idx"][tape["off"][3]: tape["off"][3] + tape["forced"][3]]
    f5 = tape["idx"][tape["off"][5]: tape["off"][5] + tape["forced"][5]]
    assert f3.tolist() == [5, 17] and f5.tolist() == [30]
    assert sum(tape["forced"]) == 3


@pytest.mark.parametrize("cell", [(0, 0), (1, 3), (3, 7), (5, 11)])
def test_drive_gradient_matches_finite_difference(cell):
    """driveSoft + soft spikes is the smooth model the drive gradient is exact for
    (src/lifdiff.js:43-53); central differences of the loss in one epoch's drive value."""
    ins, target = grad_check_inputs(seed=8)
    rng = np.random.default_rng(8)
    didx = rng.choice(ins["N"], 12, replace=False).astype(np.int32)
    prob = DiffProblem(**ins, params=dict(P0, driveSoft=True, driveEpoch=10), driveIdx=didx)
    steps = 60
    sched = rng.uniform(40, 250, (6, 12)).astype(np.float32)
    dL = np.zeros(prob.N, np.float32)
    dL[target] = 1
    sc, tape = prob.forward(steps, driveAt=sched)
    g = prob.backward(tape, dL)
    L = float(sc[target].astype(np.float64).sum())
    e, k = cell
    h = 2.0  # Hz
    up, dn = sched.copy(), sched.copy()
    up[e, k] += h
    dn[e, k] -= h
    fd = (float(prob.forward(steps, driveAt=up)[0][target].astype(np.float64).sum())
          - float(prob.forward(steps, driveAt=dn)[0][target].astype(np.float64).sum())) / (2 * h)
    ok, rel = within_tolerance(float(g["drive"][e, k]), fd, h, L)
    assert ok, (cell, float(g["drive"][e, k]), fd, rel)
    assert g["clamped"][2] == 0
