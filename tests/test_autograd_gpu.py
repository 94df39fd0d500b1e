"""The torch.autograd.Function over the adjoint: gradients with respect to per-edge gains,
per-neuron biases and per-cell-type gains of a rate-matching loss (MSE of 20 ms low-pass readout
rates against a target trace), checked against central finite differences (h = 1e-3) on 32 random
parameters. The forward pass is the smooth (soft) model, as in scripts/grad_check.mjs: finite
differences of a hard-spiking loss are meaningless. Tolerance: scripts/grad_check.mjs:98."""
import numpy as np
import pytest

from adjoint_problem import P0, grad_check_inputs, within_tolerance

pytestmark = pytest.mark.gpu
STEPS = 60


def _setup():
    import torch
    from flybrain.autograd import DiffContext
    from flybrain.diff import DiffNet
    ins, _ = grad_check_inputs(seed=11)
    N, E = ins["N"], ins["indices"].shape[0]
    rng = np.random.default_rng(11)
    cell_type = rng.integers(0, 64, N)
    data = dict(N=N, indptr=ins["indptr"], indices=ins["indices"], weights=ins["counts"], sign=ins["sign"])
    opts = dict(P0, sizeLog=ins["sizeLog"], thrMask=ins["thrMask"], biasMask=ins["biasMask"],
                logGain=ins["logGain"], thrOffset=ins["thrOffset"],
                edgeGain=np.ones(E, np.float32), bias=np.zeros(N, np.float32), outScale=np.ones(N, np.float32))
    net = DiffNet(data, opts)
    readout = np.sort(rng.choice(N, 100, replace=False))
    dctx = DiffContext(net, cell_type, readout, STEPS)
    target = torch.as_tensor(rng.uniform(0, 80, (STEPS, 100)), dtype=torch.float32, device="cuda")
    gated = np.nonzero(ins["counts"] >= P0["minSyn"])[0]
    return dctx, target, gated, rng


def _loss(dctx, target, eg, bias, tg):
    from flybrain.autograd import LIFDiffFunction, lowpass_rates
    raster = LIFDiffFunction.apply(eg, bias, tg, dctx)
    rates = lowpass_rates(raster, dctx.net.p["dt"])
    return ((rates - target) ** 2).mean()


def test_autograd_gradients_match_finite_differences():
    import torch
    dctx, target, gated, rng = _setup()
    N, E = dctx.net.N, dctx.net.E
    eg = torch.ones(E, device="cuda", requires_grad=True)
    bias = torch.zeros(N, device="cuda", requires_grad=True)
    tg = torch.as_tensor(rng.lognormal(0, 0.2, 64), dtype=torch.float32, device="cuda").requires_grad_()
    L = _loss(dctx, target, eg, bias, tg)
    L.backward()
    grads = dict(edge=eg.grad.double().cpu().numpy(), bias=bias.grad.double().cpu().numpy(),
                 type=tg.grad.double().cpu().numpy())
    picks = ([("edge", int(j)) for j in rng.choice(gated, 11, replace=False)]
             + [("bias", int(i)) for i in rng.choice(N, 11, replace=False)]
             + [("type", int(c)) for c in rng.choice(64, 10, replace=False)])
    h = 1e-3
    fails = []
    with torch.no_grad():
        base = dict(edge=eg.detach().clone(), bias=bias.detach().clone(), type=tg.detach().clone())
        for kind, idx in picks:
            vals = []
            for sgn in (1, -1):
                x = {k: v.clone() for k, v in base.items()}
                x[kind][idx] += sgn * h
                vals.append(float(_loss(dctx, target, x["edge"], x["bias"], x["type"])))
            fd = (vals[0] - vals[1]) / (2 * h)
            a = float(grads[kind][idx])
            ok, rel = within_tolerance(a, fd, h, float(L))
            if not ok:
                fails.append((kind, idx, a, fd, rel))
    assert not fails, fails
    assert np.abs(grads["edge"]).sum() > 0 and np.abs(grads["bias"]).sum() > 0 and np.abs(grads["type"]).sum() > 0


def test_first_call_after_a_drive_change_uses_its_inputs():
    """A drive change rebuilds the device network at the next forward; the edge gains, biases and
    type gains the autograd function sets must survive it (the first call's loss equals the
    second's), and so must arrays set from device tensors before a later rebuild."""
    import torch
    dctx, target, _, rng = _setup()
    net = dctx.net
    N, E = net.N, net.E
    for i in rng.choice(N, 20, replace=False):
        net.setDriveOne(int(i), 150.0)
    eg = torch.as_tensor(rng.uniform(0.5, 1.5, E), dtype=torch.float32, device="cuda")
    bias = torch.as_tensor(rng.uniform(-1, 1, N), dtype=torch.float32, device="cuda")
    tg = torch.as_tensor(rng.lognormal(0, 0.3, 64), dtype=torch.float32, device="cuda")
    with torch.no_grad():
        first = float(_loss(dctx, target, eg, bias, tg))
        second = float(_loss(dctx, target, eg, bias, tg))
    assert first == second
    # arrays set, then a drive change, then a plain forward: the rebuilt handle keeps the arrays
    sc0 = net.forward(STEPS, seed=dctx.seed, record=False).copy()
    net.setDriveOne(int(rng.integers(N)), 90.0)
    net.setDriveOne(int(rng.integers(N)), 0.0)
    net.forward(STEPS, seed=dctx.seed, record=False)
    out = tg[dctx.cell_type].contiguous()
    net.set_array("outScale", out)
    net.set_array("edgeGain", eg)
    net.set_array("bias", bias)
    sc1 = net.forward(STEPS, seed=dctx.seed, record=False)
    assert np.isfinite(sc0).all() and np.isfinite(sc1).all()
    with torch.no_grad():
        third = float(_loss(dctx, target, eg, bias, tg))
    net.setDriveOne(int(rng.integers(N)), 120.0)
    with torch.no_grad():
        fourth = float(_loss(dctx, target, eg, bias, tg))
        fifth = float(_loss(dctx, target, eg, bias, tg))
    assert fourth == fifth and np.isfinite(third)
