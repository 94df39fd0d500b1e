"""The differentiable workload at the headline scale: N=165,122 neurons, ~11M edges, 2,000 driven
neurons at 100-200 Hz, current-based, hard spikes with the fast-sigmoid surrogate of slope 25/mV
(beta 0.04), adjClip 100, checkpoints every 100 steps -- the benchmark's adjoint problem.

The GPU in the reference's arithmetic (FB_DIFF_F64) against the oracle's restatement of LIFDiff
(src/lifdiff.js:219-686) over 500 steps with a per-step loss gradient on 1,000 readout neurons:
the forward is identical (spike counts and the whole tape), and every gradient (the nine scalars,
per-neuron log-gains and biases, per-edge weights) agrees within relative 1e-5 (plus 1e-9
absolute): the two sides differ only in the order of a warp's gather sums and in the device
exp()."""
import numpy as np
import pytest

from test_adjoint_gpu import _compare_grads

pytestmark = pytest.mark.gpu

ADJ = dict(dt=0.1, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
           wSyn=0.275, coba=False, soft=False, surrogateBeta=0.04, adjClip=100.0, adaptInc=0.0, depU=0.0)


def full_problem():
    from flybrain import workload
    g, idx, hz, _ = workload("full", seed=1)
    data = dict(N=g.N, indptr=g.indptr, indices=g.indices, weights=g.counts.astype(np.float32), sign=g.sign)
    return g, idx, hz, data


@pytest.mark.slow
def test_full_scale_hard_adjoint_f64_matches_the_oracle():
    from oracle.lifdiff_oracle import DiffProblem
    from flybrain.diff import DiffNet

    g, idx, hz, data = full_problem()
    steps, K = 500, 100
    ones_e, ones_n = np.ones(g.E, np.float32), np.ones(g.N, np.float32)
    prob = DiffProblem(g.N, g.indptr, g.indices, data["weights"], g.sign, params=ADJ, driven=idx, drive_hz=hz,
                       edgeGain=ones_e, outScale=ones_n)
    net = DiffNet(data, dict(ADJ, checkpoint=K, precision="f64", edgeGain=ones_e, outScale=ones_n))
    for i, h in zip(idx.tolist(), hz.tolist()):
        net.setDriveOne(i, h)
    sc0, tape = prob.forward(steps, seed=3, checkpoint=K)
    sc1 = net.forward(steps, seed=3)
    assert sc0.tobytes() == sc1.tobytes()
    off, ix, amp = net.tape()
    np.testing.assert_array_equal(off, tape["off"])
    np.testing.assert_array_equal(ix, tape["idx"])
    np.testing.assert_array_equal(amp, tape["amp"])
    assert tape["forced"].sum() > 1000

    rng = np.random.default_rng(3)
    readout = np.sort(rng.choice(g.N, 1000, replace=False)).astype(np.int32)
    dro = (rng.standard_normal((steps, readout.shape[0])) * 1e-3).astype(np.float32)
    dL = np.zeros((steps, g.N), np.float32)
    dL[:, readout] = dro
    g0 = prob.backward(tape, dL)
    g1 = net.backward(dro, readout=readout)
    assert np.isfinite(g1["edge"]).all() and np.abs(g1["edge"]).sum() > 0
    _compare_grads(g0, g1)
