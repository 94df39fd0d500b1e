"""Gradient accuracy at the headline scale: the differentiable workload (N=165,122, ~11M edges,
2,000 driven neurons, current-based, 500 steps at dt 0.1 ms, checkpoints every 100) in its smooth
form -- soft spikes with the fast-sigmoid slope of 25/mV (beta 0.04) -- through the autograd
function, with per-edge gains, per-neuron biases and 64 cell-type gains as inputs and the MSE of
20 ms low-pass rates of 1,000 readouts against a 0-80 Hz target as the loss. 32 parameters (11
edges, 11 biases, 10 types, drawn among those with a non-zero gradient) are checked against
central finite differences (h = 1e-3) of the forward in double (FP64 finite differences), with the
adjoint in double and in float32: every row within scripts/grad_check.mjs's tolerance, and the
relative errors stated by the test's output."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 500


def _context(prec):
    import torch
    from flybrain.autograd import DiffContext
    from flybrain.diff import DiffNet
    from test_adjoint_scale_gpu import ADJ, full_problem
    g, idx, hz, data = full_problem()
    rng = np.random.default_rng(3)
    net = DiffNet(data, dict(ADJ, soft=True, checkpoint=100, precision=prec, edgeGain=np.ones(g.E, np.float32),
                             bias=np.zeros(g.N, np.float32), outScale=np.ones(g.N, np.float32)))
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
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_full_scale_soft_gradients_match_fp64_finite_differences(prec):
    from flybrain.autograd import finite_difference_check
    dctx, target, eg, bias, tg = _context(prec)
    r = finite_difference_check(dctx, target, eg, bias, tg, seed=5, fd_precision="f64")
    print(f"{prec} adjoint vs FP64 FD on {r['params']} parameters: max rel {r['max_rel']:.3g}, "
          f"median rel {r['median_rel']:.3g}, {r['passed']} within grad_check's tolerance")
    for row in r["rows"]:
        print("  ", row)
    assert r["params"] == 32
    assert r["passed"] == r["params"], [x for x in r["rows"] if not x["ok"]]
