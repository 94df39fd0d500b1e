"""Gradient accuracy at the headline scale: the differentiable workload's network (N=165,122,
~11M edges, 2,000 driven neurons at 100-200 Hz, current-based, checkpoints every 100), 500 steps at
dt 0.1 ms, in the smooth form scripts/grad_check.mjs checks -- soft spikes with its surrogate width
of 1.5 mV and no adjoint clipping (clipping is a deliberate bound for hard spikes, not part of the
gradient) -- through the autograd function, with per-edge gains, per-neuron biases and 64 cell-type
gains as inputs and the MSE of 20 ms low-pass rates of 1,000 readouts against a 0-80 Hz target as
the loss, evaluated in float64.

With the benchmark's steep surrogate (25/mV) the smooth model is nearly silent at rest: no
parameter moves the loss within float32 resolution and every central difference is exactly 0, so
that setting cannot be checked this way.

32 parameters (11 edges, 11 biases, 10 types, drawn among the 44, 44 and 40 with the largest
gradients) are checked against central finite differences of the forward in double (FP64 finite
differences). Steps: 4e-3 for a type gain, 4e-2 for an edge gain, 0.4 mV for a bias. The
network state is float32 (as the reference's Float32Array state) and spikes below 1e-4 stay off the
tape, so a difference carries noise of a fixed size in the loss, and its relative error falls as
the step grows: over these 32 parameters the largest error is 6.1e-3 at a quarter of these steps,
4.7e-3 at half, 1.4e-3 at these, and twice these steps give errors of the same size (the
curvature of the loss does not show yet; scripts/grad_check.mjs:82-86 sizes its steps per
parameter for the same reason). Both the double-precision and the float32 adjoint must agree with every difference within
0.3% and with the median within 0.1%; the measured errors are printed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 500
H = dict(edge=4e-2, bias=0.4, type=4e-3)


def _context(prec, problem=None):
    import torch
    from flybrain.autograd import DiffContext
    from flybrain.diff import DiffNet
    from test_adjoint_scale_gpu import ADJ, full_problem
    g, idx, hz, data = problem or full_problem()
    rng = np.random.default_rng(3)
    net = DiffNet(data, dict(ADJ, soft=True, surrogateBeta=1.5, adjClip=0.0, checkpoint=100, precision=prec,
                             edgeGain=np.ones(g.E, np.float32), bias=np.zeros(g.N, np.float32),
                             outScale=np.ones(g.N, np.float32)))
    for i, h in zip(idx.tolist(), hz.tolist()):
        net.setDriveOne(i, h)
    readout = np.sort(rng.choice(g.N, 1000, replace=False))
    dctx = DiffContext(net, g.cell_type, readout, STEPS, seed=3)
    target = torch.as_tensor(rng.uniform(0, 80, (1, 1000)), dtype=torch.float32, device="cuda")
    eg = torch.ones(g.E, device="cuda", requires_grad=True)
    bias = torch.zeros(g.N, device="cuda", requires_grad=True)
    tg = torch.as_tensor(rng.lognormal(0, 0.2, 64), dtype=torch.float32, device="cuda").requires_grad_()
    return dctx, target, eg, bias, tg


@pytest.mark.slow
def test_full_scale_soft_gradients_match_fp64_finite_differences():
    from flybrain.autograd import finite_difference_check
    from test_adjoint_scale_gpu import full_problem
    prob = full_problem()
    dctx, target, eg, bias, tg = _context("f64", prob)
    ctx32 = _context("f32", prob)[0]
    r = finite_difference_check(dctx, target, eg, bias, tg, h=H, seed=5, fd_precision="f64", others={"f32": ctx32})
    print(f"\nf64 adjoint vs FP64 FD on {r['params']} parameters: max rel {r['max_rel']:.3g}, median "
          f"{r['median_rel']:.3g}; per kind {r['per_kind']}; f32 adjoint: {r['others']['f32']}")
    for row in r["rows"]:
        print("  ", {k: (round(v, 6) if isinstance(v, float) else v) for k, v in row.items()})
    assert r["params"] == 32
    assert all(x["fd"] != 0 for x in r["rows"]), "a finite difference is 0: the check has no signal"
    for row in r["rows"]:
        assert row["rel"] <= 3e-3 and row["rel_f32"] <= 3e-3, row
    assert r["median_rel"] <= 1e-3 and r["others"]["f32"]["median_rel"] <= 1e-3, r
