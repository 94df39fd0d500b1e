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


def lowpass_rates(raster: torch.Tensor, dt_ms: float, tau_ms: float = 20.0, dtype=None) -> torch.Tensor:
    """Exponentially low-passed firing rates in Hz of a (steps x R) spike raster, exactly:
    r_t = a r_{t-1} + c s_t with a = exp(-dt / tau), c = (1 - a) / dt (dt in s), r_{-1} = 0.
    Evaluated blockwise in float64 as r_t = a^(t+1) r_start + c a^t sum_{k<=t} a^-k s_k, with
    blocks short enough that a^-k stays below 1e12; differentiable through torch ops. The result
    has the raster's dtype unless `dtype` is given (torch.float64 keeps the double rates)."""
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
    return torch.cat(out).to(dtype or raster.dtype)


def rate_loss(dctx: DiffContext, target: torch.Tensor, edge_gain, bias, type_gain, dtype=None) -> torch.Tensor:
    """MSE between the 20 ms low-pass rates of the readout raster and a target trace (in `dtype`,
    default the raster's float32)."""
    raster = LIFDiffFunction.apply(edge_gain, bias, type_gain, dctx)
    r = lowpass_rates(raster, dctx.net.p["dt"], dtype=dtype)
    return ((r - target.to(r.dtype)) ** 2).mean()


def adjoint_gradients(dctx: DiffContext, target, edge_gain, bias, type_gain) -> dict:
    """The adjoint's gradients of rate_loss (in float64) for the three inputs, as float64 numpy
    arrays, and the loss."""
    e = edge_gain.detach().clone().requires_grad_()
    b = bias.detach().clone().requires_grad_()
    t = type_gain.detach().clone().requires_grad_()
    L = rate_loss(dctx, target, e, b, t, dtype=torch.float64)
    L.backward()
    return dict(edge=e.grad.double().cpu().numpy(), bias=b.grad.double().cpu().numpy(),
                type=t.grad.double().cpu().numpy(), loss=float(L.detach()))


def finite_difference_check(dctx: DiffContext, target, edge_gain, bias, type_gain, n_edge=11, n_bias=11,
                            n_type=10, h=1e-3, seed=0, fd_precision="f64", pool=4, others=None):
    """The adjoint's gradients of rate_loss (evaluated in float64) against central finite
    differences, the check of scripts/grad_check.mjs:69-109 applied to the three input kinds of
    LIFDiffFunction.

    Parameters of each kind are drawn at random among the pool * n of that kind with the largest
    adjoint gradients: in a large, sparsely active network most gradients are zero or far below
    what a central difference can resolve (the difference is then exactly 0 and the check says
    nothing), so the check is made where the loss actually responds. The adjoint runs in the
    context's precision; each finite difference takes two forward passes in `fd_precision`
    ("f64": double-precision finite differences). h is one step for every kind, or a dict
    {"edge": .., "bias": .., "type": ..}: the network's state is float32 (as the reference's
    Float32Array state), so a kind whose perturbation moves the loss by less than about 1e-6 of
    itself is measured by rounding noise rather than slope and needs a larger step
    (scripts/grad_check.mjs:82-86 picks its steps per parameter for the same reason). A row also
    records grad_check's tolerance |g - fd| <= 1e-3 |fd| + 4e-6 |L| / h (scripts/grad_check.mjs:98).
    Returns the rows and the maximum and median relative errors |g - fd| / |fd|. others: named
    further contexts (the same network in another arithmetic, say) whose adjoints are compared
    with the same finite differences (row fields rel_<name>, summary others[<name>])."""
    f64 = torch.float64
    for p in (edge_gain, bias, type_gain):
        p.grad = None
    L = rate_loss(dctx, target, edge_gain, bias, type_gain, dtype=f64)
    L.backward()
    grads = dict(edge=edge_gain.grad.double().cpu().numpy(), bias=bias.grad.double().cpu().numpy(),
                 type=type_gain.grad.double().cpu().numpy())
    rng = np.random.default_rng(seed)

    def pick(kind, n):
        a = np.abs(grads[kind])
        top = np.argsort(-a, kind="stable")[: min(pool * n, int((a > 0).sum()))]
        return [(kind, int(i)) for i in rng.choice(top, min(n, top.shape[0]), replace=False)]

    picks = pick("edge", n_edge) + pick("bias", n_bias) + pick("type", n_type)
    base = dict(edge=edge_gain.detach().clone(), bias=bias.detach().clone(), type=type_gain.detach().clone())
    adj_prec = dctx.over.get("precision", dctx.net.p["precision"])
    saved = dict(dctx.over)
    dctx.over["precision"] = fd_precision
    rows = []
    try:
        with torch.no_grad():
            Lfd = float(rate_loss(dctx, target, base["edge"], base["bias"], base["type"], dtype=f64))
            for kind, idx in picks:
                hk = float(h[kind]) if isinstance(h, dict) else float(h)
                vals = []
                for sgn in (1, -1):
                    x = {k: v.clone() for k, v in base.items()}
                    x[kind][idx] += sgn * hk
                    vals.append(float(rate_loss(dctx, target, x["edge"], x["bias"], x["type"], dtype=f64)))
                fd = (vals[0] - vals[1]) / (2 * hk)
                a = float(grads[kind][idx])
                ok = abs(a - fd) <= 1e-3 * abs(fd) + 4e-6 * abs(Lfd) / hk
                rows.append(dict(kind=kind, index=idx, h=hk, adjoint=a, fd=fd, rel=abs(a - fd) / max(abs(fd), 1e-300),
                                 ok=ok))
    finally:
        dctx.over.clear()
        dctx.over.update(saved)
    extra = {}
    for name, ctx2 in (others or {}).items():
        g2 = adjoint_gradients(ctx2, target, base["edge"], base["bias"], base["type"])
        rel2 = []
        for r in rows:
            a2 = float(g2[r["kind"]][r["index"]])
            r["adjoint_" + name] = a2
            r["rel_" + name] = abs(a2 - r["fd"]) / max(abs(r["fd"]), 1e-300)
            rel2.append(r["rel_" + name])
        rel2 = np.array(rel2) if rel2 else np.zeros(1)
        extra[name] = dict(max_rel=float(rel2.max()), median_rel=float(np.median(rel2)))
    rel = np.array([r["rel"] for r in rows]) if rows else np.zeros(1)
    per_kind = {}
    for k in ("edge", "bias", "type"):
        rk = np.array([r["rel"] for r in rows if r["kind"] == k])
        if rk.size:
            per_kind[k] = dict(max_rel=float(rk.max()), median_rel=float(np.median(rk)), n=int(rk.size))
    return dict(h=h, adjoint_precision=adj_prec, fd_precision=fd_precision, loss=float(L.detach()),
                params=len(rows), passed=int(sum(r["ok"] for r in rows)), max_rel=float(rel.max()),
                median_rel=float(np.median(rel)), per_kind=per_kind, others=extra, rows=rows)
