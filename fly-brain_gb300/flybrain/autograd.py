"""torch.autograd.Function over the differentiable brain (fb_diff_*).

LIFDiffFunction.apply(edge_gain, bias, type_gain, ctx) runs the LIFDiff forward pass on the GPU
with per-edge gains (edgeGain, src/lifdiff.js:128-131), an additive per-neuron bias current and
per-cell-type gains on outgoing synapses (outScale = type_gain[cell_type], the role typeGains
plays in src/brainmodel.js:63-100), and returns the spike raster of the readout neurons
(steps x R, spike amplitudes). Its backward runs the adjoint (src/lifdiff.js:494-686) with the
raster's gradient as the per-step dLoss/dspike and returns gradients for all three inputs.
"""
from __future__ import annotations

import numpy as np
import torch

from .diff import DiffNet


class DiffContext:
    """What the function needs besides its differentiable inputs: the network, the cell type of
    each neuron, the readout set, the window and the seed."""

    def __init__(self, net: DiffNet, cell_type, readout, steps: int, seed: int = 1, **over):
        self.net = net
        self.cell_type_np = np.asarray(cell_type, np.int64)
        self.cell_type = torch.as_tensor(self.cell_type_np, device="cuda")
        self.readout = np.ascontiguousarray(readout, np.int32)
        self.steps = int(steps)
        self.seed = int(seed)
        self.over = over
        # dW_j / d edgeGain_j = count_j * inScale[post] * (inhGain if the presynaptic sign < 0)
        p = dict(net.p, **over)
        pre = np.repeat(np.arange(net.N), np.diff(net.indptr.astype(np.int64)))
        inh = net.sign[pre] < 0
        ins = net.arrays.get("in_scale")
        if ins is None:
            sl = net.arrays.get("size_log")
            sl = np.zeros(net.N, np.float32) if sl is None else sl
            ins = np.minimum(p["boostCap"], np.maximum(1 / p["maxSizeScale"],
                                                       np.exp(-p["sizeAlpha"] * sl.astype(np.float64))))
            ins = ins.astype(np.float32).astype(np.float64)
        dw = net.counts.astype(np.float64) * np.asarray(ins, np.float64)[net.indices]
        dw[inh] *= p["inhGain"]
        self.dW_dgain = torch.as_tensor(dw, device="cuda")


class LIFDiffFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, edge_gain, bias, type_gain, dctx: DiffContext):
        net = dctx.net
        eg = edge_gain.detach().float().contiguous()
        bs = bias.detach().float().contiguous()
        out_scale = type_gain.detach().float()[dctx.cell_type].contiguous()
        torch.cuda.synchronize()  # the library copies on its own stream
        net.set_array("edgeGain", eg)
        net.set_array("bias", bs)
        net.set_array("outScale", out_scale)
        net.forward(dctx.steps, seed=dctx.seed, record=True, **dctx.over)
        raster = torch.zeros((dctx.steps, dctx.readout.shape[0]), dtype=torch.float32, device="cuda")
        net.raster(dctx.readout, out=raster)
        ctx.dctx = dctx
        ctx.ntypes = type_gain.shape[0]
        return raster

    @staticmethod
    def backward(ctx, g_raster):
        dctx = ctx.dctx
        gr = g_raster.detach().float().contiguous()
        torch.cuda.synchronize()
        dev = g_raster.device
        g = dctx.net.backward(gr, readout=dctx.readout, device=dev)
        g_edge = g["edge"] * dctx.dW_dgain
        g_bias = g["bias"]
        # per-type sums in neuron order on the host (a deterministic order; device scatter-adds
        # are not)
        g_type = torch.as_tensor(np.bincount(dctx.cell_type_np, weights=g["outScale"].cpu().numpy(),
                                             minlength=ctx.ntypes), device=dev)
        return g_edge.float(), g_bias.float(), g_type.float(), None


def lowpass_rates(raster: torch.Tensor, dt_ms: float, tau_ms: float = 20.0) -> torch.Tensor:
    """Exponentially low-passed firing rates in Hz of a (steps x R) spike raster, exactly:
    r_t = a r_{t-1} + c s_t with a = exp(-dt / tau), c = (1 - a) / dt (dt in s), r_{-1} = 0.
    Evaluated blockwise in float64 as r_t = a^(t+1) r_start + c a^t sum_{k<=t} a^-k s_k, with
    blocks short enough that a^-k stays below 1e12; differentiable through torch ops."""
    a = float(np.exp(-dt_ms / tau_ms))
    c = (1 - a) / (dt_ms / 1000.0)
    T, R = raster.shape
    block = max(1, min(T, int(27.0 * tau_ms / dt_ms)))
    x = raster.to(torch.float64)
    k = torch.arange(block, dtype=torch.float64, device=raster.device)
    up, down = a ** (-k), a ** k
    r = torch.zeros(R, dtype=torch.float64, device=raster.device)
    out = []
    for b0 in range(0, T, block):
        xb = x[b0:b0 + block]
        n = xb.shape[0]
        cs = torch.cumsum(xb * up[:n, None], 0)
        rb = (a * down[:n, None]) * r[None, :] + c * down[:n, None] * cs
        out.append(rb)
        r = rb[-1]
    return torch.cat(out).to(raster.dtype)
