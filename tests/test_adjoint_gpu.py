"""The differentiable brain step and its adjoint on the GPU (fb_diff_*) against the oracle's
restatement of LIFDiff, and against central finite differences of the GPU's own forward pass.

Tolerances: both sides compute in double with float32 state and the same per-target summation
order, so the hard-spike forward is bit-identical (tape and spike counts); gradients differ only
by summation order of a warp's gather and of per-target inScale sums (double vs the reference's
float32) and by the device exp(): relative 1e-5 (plus 1e-9 absolute). Finite differences use the
tolerance of scripts/grad_check.mjs:98."""
import numpy as np
import pytest

from adjoint_problem import H, P0, grad_check_inputs, within_tolerance

pytestmark = pytest.mark.gpu
REL, ABS = 1e-5, 1e-9


def _pair(ins, params, driven=None, hz=None):
    from oracle.lifdiff_oracle import DiffProblem
    from flybrain.diff import DiffNet
    prob = DiffProblem(**ins, params=params, driven=driven, drive_hz=hz)
    data = dict(N=ins["N"], indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"])
    opts = dict(params)
    for k_src, k_dst in (("sizeLog", "sizeLog"), ("thrMask", "thrMask"), ("biasMask", "biasMask"),
                         ("logGain", "logGain"), ("outScale", "outScale"), ("thrOffset", "thrOffset")):
        if ins.get(k_src) is not None:
            opts[k_dst] = ins[k_src]
    net = DiffNet(data, opts)
    if driven is not None:
        for i, h in zip(driven, hz):
            net.setDriveOne(int(i), float(h))
    return prob, net


def _close(a, b, rel=REL, abs_=ABS):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    same = (a == b) | (np.isnan(a) & np.isnan(b))  # non-finite entries must agree exactly
    with np.errstate(invalid="ignore"):
        near = np.abs(a - b) <= rel * np.maximum(np.abs(a), np.abs(b)) + abs_
    return bool(np.all(same | near))


def _compare_grads(g0, g1, E_check=True):
    for k, v in g0["params"].items():
        assert _close(v, g1["params"][k]), (k, v, g1["params"][k])
    assert _close(g0["logGain"], g1["logGain"], abs_=1e-7)
    assert _close(g0["gBias"], g1["bias"])
    if E_check:
        assert _close(g0["gEdge"], g1["edge"], abs_=1e-9)


def test_soft_gradients_match_oracle():
    ins, target = grad_check_inputs()
    prob, net = _pair(ins, P0)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    sc0, tape = prob.forward(60)
    g0 = prob.backward(tape, dL)
    sc1 = net.forward(60)
    assert _close(sc0, sc1, rel=1e-6)
    g1 = net.backward(dL)
    _compare_grads(g0, g1)


@pytest.mark.parametrize("name", ["wSyn", "vThresh", "depU", "sizeAlpha"])
def test_soft_gradient_matches_gpu_finite_difference(name):
    ins, target = grad_check_inputs()
    _, net = _pair(ins, P0)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    L = float(net.forward(60)[target].astype(np.float64).sum())
    g = net.backward(dL)["params"][name]
    h = H[name]
    lp = float(net.forward(60, record=False, **{name: P0[name] + h})[target].astype(np.float64).sum())
    lm = float(net.forward(60, record=False, **{name: P0[name] - h})[target].astype(np.float64).sum())
    fd = (lp - lm) / (2 * h)
    ok, rel = within_tolerance(g, fd, h, L)
    assert ok, (name, g, fd, rel)


def _hard_inputs():
    ins, target = grad_check_inputs(seed=7)
    ins["logGain"] = np.zeros(ins["N"], np.float32)  # exp(0) = 1 exactly on both sides
    rng = np.random.default_rng(7)
    driven = rng.choice(ins["N"], 40, replace=False).astype(np.int32)
    hz = rng.uniform(50, 250, 40)
    # the hard-spike adjoint grows exponentially on this very active recurrent subgraph (about
    # 1e8 after 120 steps with beta = 2; with the fast-sigmoid slope 25/mV, beta = 0.04, it
    # overflows within a few hundred steps, identically on both sides): comparisons of finite
    # gradients use beta = 2 over 120 steps
    params = dict(coba=True, soft=False, surrogateBeta=2.0, wSyn=0.5, minSyn=3.0, adaptInc=0.3,
                  depU=0.1, laminaBias=9.0, kcThreshold=2.0, inhGain=0.8, sizeAlpha=0.5, checkpoint=16)
    return ins, target, driven, hz, params


def test_hard_forward_tape_is_identical_to_oracle():
    ins, target, driven, hz, params = _hard_inputs()
    prob, net = _pair(ins, params, driven, hz)
    sc0, tape = prob.forward(400, seed=3)
    sc1 = net.forward(400, seed=3)
    off, idx, amp = net.tape()
    np.testing.assert_array_equal(off, tape["off"])
    np.testing.assert_array_equal(idx, tape["idx"])
    np.testing.assert_array_equal(amp, tape["amp"])
    assert sc0.tobytes() == sc1.tobytes()
    assert tape["forced"].sum() > 0 and idx.shape[0] > 1000


def test_hard_gradients_match_oracle():
    ins, target, driven, hz, params = _hard_inputs()
    prob, net = _pair(ins, params, driven, hz)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    _, tape = prob.forward(120, seed=3)
    g0 = prob.backward(tape, dL)
    net.forward(120, seed=3)
    g1 = net.backward(dL)
    assert all(np.isfinite(v) for v in g1["params"].values()) and np.isfinite(g1["edge"]).all()
    _compare_grads(g0, g1)


@pytest.mark.parametrize("delay", [0.1, 0.2, 0.3])
def test_short_delays_match_oracle(delay):
    """Delays of one to three steps: with one step (two ring slots) a delivery reads the tape the
    step before wrote, so the forward keeps the tape write ahead of the next delivery; with more
    the two overlap. Tape, spike counts and gradients against the oracle, hard spikes."""
    ins, target, driven, hz, params = _hard_inputs()
    params = dict(params, delay=delay)
    prob, net = _pair(ins, params, driven, hz)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    sc0, tape = prob.forward(120, seed=3)
    sc1 = net.forward(120, seed=3)
    assert sc0.tobytes() == sc1.tobytes()
    off, idx, amp = net.tape()
    np.testing.assert_array_equal(off, tape["off"])
    np.testing.assert_array_equal(idx, tape["idx"])
    assert idx.shape[0] > 300
    _compare_grads(prob.backward(tape, dL), net.backward(dL))


def test_captured_passes_follow_a_delay_change():
    """Forward passes of one network with the delay alternating between one and three steps:
    each pass's graph is keyed on the ring depth (the stream order differs), so every pass matches
    the oracle at its own delay, the cached ones included."""
    from oracle.lifdiff_oracle import DiffProblem
    ins, target, driven, hz, params = _hard_inputs()
    _, net = _pair(ins, params, driven, hz)
    probs = {d: DiffProblem(**ins, params=dict(params, delay=d), driven=driven, drive_hz=hz) for d in (0.1, 0.3)}
    for delay in (0.1, 0.3, 0.1, 0.3):
        sc0, tape = probs[delay].forward(100, seed=3)
        sc1 = net.forward(100, seed=3, delay=delay)
        assert sc0.tobytes() == sc1.tobytes(), delay
        off, idx, _ = net.tape()
        np.testing.assert_array_equal(off, tape["off"])
        np.testing.assert_array_equal(idx, tape["idx"])


def test_steep_surrogate_nonfinite_values_agree():
    """With the steep surrogate the adjoint overflows; both sides zero and count the same
    non-finite gradients (src/lifdiff.js:681-684)."""
    ins, target, driven, hz, params = _hard_inputs()
    prob, net = _pair(ins, dict(params, surrogateBeta=0.04), driven, hz)
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    _, tape = prob.forward(400, seed=3)
    g0 = prob.backward(tape, dL)
    net.forward(400, seed=3)
    g1 = net.backward(dL)
    assert g1["clamped"]["params"] == g0["clamped"][0] and g1["clamped"]["logGain"] == g0["clamped"][1]
    _compare_grads(g0, g1)


def test_readout_loss_truncation_clip_current_based():
    """Per-step loss over a readout set, lossFrom, truncated BPTT and the adjoint clip, with the
    current-based membrane."""
    ins, target, driven, hz, params = _hard_inputs()
    params = dict(params, coba=False, adjClip=5.0, checkpoint=25)
    prob, net = _pair(ins, params, driven, hz)
    steps = 160
    rng = np.random.default_rng(1)
    readout = np.sort(rng.choice(ins["N"], 50, replace=False)).astype(np.int32)
    dLro = rng.normal(0, 1, (steps, readout.shape[0])).astype(np.float32)
    dense = np.zeros((steps, ins["N"]), np.float32)
    dense[:, readout] = dLro
    _, tape = prob.forward(steps, seed=5, checkpoint=25)
    g0 = prob.backward(tape, dense, truncate=40, lossFrom=20)
    net.forward(steps, seed=5)
    g1 = net.backward(dLro, truncate=40, lossFrom=20, readout=readout)
    _compare_grads(g0, g1)
    r = net.raster(readout)
    off, idx, amp = net.tape()
    t = int(np.argmax([off[k + 1] - off[k] for k in range(steps)]))
    for i, a in zip(idx[off[t]:off[t + 1]], amp[off[t]:off[t + 1]]):
        if i in set(readout.tolist()):
            assert r[t, int(np.searchsorted(readout, i))] == a


# ---- float32 arithmetic (precision="f32"): the same expressions with float intermediates ----

def _rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(1e-30, float(np.max(np.abs(b)))))


@pytest.mark.parametrize("name", ["wSyn", "vThresh", "depU", "sizeAlpha", "eInh", "laminaBias"])
def test_f32_soft_gradient_matches_gpu_finite_difference(name):
    """Float intermediates keep the adjoint within scripts/grad_check.mjs:98's tolerance of central
    differences of the float forward."""
    ins, target = grad_check_inputs()
    _, net = _pair(ins, dict(P0, precision="f32"))
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    L = float(net.forward(60)[target].astype(np.float64).sum())
    g = net.backward(dL)["params"][name]
    h = H[name]
    lp = float(net.forward(60, record=False, **{name: P0[name] + h})[target].astype(np.float64).sum())
    lm = float(net.forward(60, record=False, **{name: P0[name] - h})[target].astype(np.float64).sum())
    fd = (lp - lm) / (2 * h)
    ok, rel = within_tolerance(g, fd, h, L)
    assert ok, (name, g, fd, rel)


def test_f32_soft_gradients_track_f64():
    """Soft spikes: the float pass follows the double one; every scalar, per-neuron and per-edge
    gradient agrees to 1e-3 of its vector's largest entry."""
    ins, target = grad_check_inputs()
    dL = np.zeros(ins["N"], np.float32)
    dL[target] = 1
    out = {}
    for prec in ("f64", "f32"):
        _, net = _pair(ins, dict(P0, precision=prec))
        sc = net.forward(60)
        out[prec] = (sc, net.backward(dL))
    (sc64, g64), (sc32, g32) = out["f64"], out["f32"]
    assert _rel_err(sc32, sc64) < 1e-4
    for k in g64["params"]:
        assert abs(g32["params"][k] - g64["params"][k]) <= 1e-3 * abs(g64["params"][k]) + 1e-9, k
    assert _rel_err(g32["logGain"], g64["logGain"]) < 1e-3
    assert _rel_err(g32["bias"], g64["bias"]) < 1e-3
    assert _rel_err(g32["edge"], g64["edge"]) < 1e-3
    assert _rel_err(g32["outScale"], g64["outScale"]) < 1e-3


def test_f32_hard_forward_tracks_f64():
    """Hard spikes: a threshold crossing can flip when float rounding moves v across it; over
    400 steps of the driven subgraph the spike totals agree to 2% and the forced spikes (the
    random draws) of the first steps are identical."""
    ins, target, driven, hz, params = _hard_inputs()
    tapes = {}
    for prec in ("f64", "f32"):
        _, net = _pair(ins, dict(params, precision=prec), driven, hz)
        sc = net.forward(400, seed=3)
        tapes[prec] = (sc, net.tape())
    (sc64, (o64, i64, _)), (sc32, (o32, i32, _)) = tapes["f64"], tapes["f32"]
    assert abs(float(sc32.sum()) - float(sc64.sum())) <= 0.02 * float(sc64.sum())
    np.testing.assert_array_equal(i32[: o32[5]], i64[: o64[5]])


def test_precision_is_validated():
    from flybrain._native import FlyBrainError
    ins, _ = grad_check_inputs()
    _, net = _pair(ins, P0)
    with pytest.raises(ValueError):
        net.forward(4, precision="f16")
    q = net.params()
    q.precision = 7
    import ctypes as C
    sc = np.zeros(ins["N"], np.float32)
    with pytest.raises(FlyBrainError):
        from flybrain import _native as nat
        nat.check(net.L.fb_diff_forward(net.h, C.byref(q), 4, 1, 0, sc.ctypes.data))
