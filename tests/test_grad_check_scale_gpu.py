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
differences). Steps: 1e-3 for the type gains; 1e-2 for an edge gain and 1e-1 mV for a bias, whose
single-parameter perturbations otherwise move the loss by less than the float32 state resolves
(scripts/grad_check.mjs:82-86 sizes its steps for the same reason). Both the double-precision and
the float32 adjoint must agree with every difference within 1%, the type gains within 0.3%; the
measured errors are printed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 500
H = dict(edge=1e-2, bias=1e-1, type=1e-3)


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
        bound = 3e-3 if row["kind"] == "type" else 1e-2
        assert row["rel"] <= bound and row["rel_f32"] <= bound, row
