"""The differentiable brain on the GB300 kernels: a drop-in for the reference's LIFDiff
(src/lifdiff.js:77-687) -- new LIFDiff(data, opts), setDrive/setDriveOne, forward(steps,
{seed, record}) and backward(tape, dLdSpike, {truncate, lossFrom}) returning
{params, logGain, clamped} -- plus per-edge, per-neuron-bias and outScale gradients, and a
torch.autograd.Function over per-edge gains, per-neuron biases and per-cell-type gains.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat

DIFF_PARAMS = ["wSyn", "sizeAlpha", "inhGain", "eInh", "vThresh", "kcThreshold", "laminaBias",
               "adaptInc", "depU"]  # src/lifdiff.js:75
EXC_SIGN = np.array([0, 1, -1, -1, 1, 1, 1, -1], np.float32)  # src/lif.js:5

# src/lifdiff.js:86-109
DIFF_DEFAULTS = dict(
    dt=0.5, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
    wSyn=0.3, adaptInc=0.0, adaptTau=100.0, depU=0.0, depTau=200.0, minSyn=1.0, coba=True,
    eExc=0.0, eInh=-70.0, inhGain=1.0, sizeAlpha=0.0, maxSizeScale=20.0, boostCap=1.0,
    kcThreshold=0.0, laminaBias=0.0, surrogateBeta=2.0, adjClip=0.0, soft=False, checkpoint=16,
    precision="f64",
)
PRECISIONS = dict(f64=0, f32=1)

_ARRAYS_N = ("size_log", "in_scale", "log_gain", "out_scale", "thr_offset", "beta", "bias")
_MASKS = ("thr_mask", "bias_mask", "sensory")
_FIELDS = dict(log_gain=0, out_scale=1, thr_offset=2, bias=3, edge_gain=4, drive=5)


def make_params(p: dict) -> nat.FbDiffParams:
    q = nat.FbDiffParams()
    for k, _ in nat.FbDiffParams._fields_:
        if k in ("coba", "soft", "checkpoint", "precision"):
            continue
        setattr(q, k, float(p[k]))
    q.coba, q.soft, q.checkpoint = int(bool(p["coba"])), int(bool(p["soft"])), int(p["checkpoint"])
    if p["precision"] not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, not {p['precision']!r}")
    q.precision = PRECISIONS[p["precision"]]
    return q


class DiffNet:
    """LIFDiff on the device. data: {N, indptr, indices, weights (raw counts), nt} as the
    reference takes it (or sign= for preSign); opts: model parameters and per-neuron structure
    (sizeLog, thrMask, biasMask, logGain, outScale, thrOffset, sensoryMask, edgeGain, inScale,
    surrogateBeta as an array, bias)."""

    def __init__(self, data: dict, opts: dict | None = None, tape_cap: int = 0):
        self.L = nat.load()
        opts = dict(opts or {})
        self.N = int(data["N"])
        self.indptr = np.ascontiguousarray(data["indptr"], np.uint32)
        self.indices = np.ascontiguousarray(data["indices"], np.uint32)
        self.counts = np.ascontiguousarray(data["weights"], np.float32)
        self.E = int(self.indices.shape[0])
        if opts.get("preSign") is not None:
            self.sign = np.ascontiguousarray(opts["preSign"], np.float32)
        elif data.get("sign") is not None:
            self.sign = np.ascontiguousarray(data["sign"], np.float32)
        else:
            self.sign = EXC_SIGN[np.asarray(data["nt"])]
        self.p = dict(DIFF_DEFAULTS)
        for k in list(opts):
            if k in DIFF_DEFAULTS and not isinstance(opts[k], np.ndarray):
                self.p[k] = opts[k]
        beta = opts.get("surrogateBeta")
        self.arrays = dict(
            size_log=opts.get("sizeLog"), in_scale=opts.get("inScale"), log_gain=opts.get("logGain"),
            out_scale=opts.get("outScale"), thr_offset=opts.get("thrOffset"),
            beta=beta if isinstance(beta, np.ndarray) else None, bias=opts.get("bias"),
            thr_mask=opts.get("thrMask"), bias_mask=opts.get("biasMask"), sensory=opts.get("sensoryMask"),
            edge_gain=opts.get("edgeGain"))
        self.drive = np.zeros(self.N, np.float32)
        self.drivenSet: dict[int, None] = {}
        self._keep = []
        self.h = None
        self._create(tape_cap)

    def _create(self, tape_cap):
        net = nat.FbDiffNet()
        net.N, net.E = self.N, self.E
        keep = []

        def arr(x, dt):
            if x is None:
                return None
            a = np.ascontiguousarray(x, dt)
            keep.append(a)
            return a.ctypes.data

        net.indptr, net.indices = arr(self.indptr, np.uint32), arr(self.indices, np.uint32)
        net.counts, net.sign = arr(self.counts, np.float32), arr(self.sign, np.float32)
        for k in _ARRAYS_N + ("edge_gain",):
            setattr(net, k, arr(self.arrays[k], np.float32))
        for k in _MASKS:
            setattr(net, k, arr(self.arrays[k], np.uint8))
        driven = np.array(list(self.drivenSet), np.int32)
        net.nDriven = int(driven.shape[0])
        net.drive = arr(self.drive, np.float32)
        net.driven = arr(driven if driven.shape[0] else np.zeros(1, np.int32), np.int32)
        h = C.c_void_p()
        nat.check(self.L.fb_diff_create(C.byref(net), int(tape_cap), C.byref(h)))
        if self.h:
            self.L.fb_diff_destroy(self.h)
        self.h = h
        self._tape_cap = tape_cap
        self._drive_dirty = False

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.fb_diff_destroy(h)
            self.h = None

    # src/lifdiff.js:202-207: the driven set keeps insertion order, which fixes the draw order
    def setDriveOne(self, i, rate):
        i = int(i)
        self.drive[i] = rate
        if rate > 0:
            self.drivenSet.setdefault(i, None)
        else:
            self.drivenSet.pop(i, None)
        self._drive_dirty = True

    def setDrive(self, ix, rate):
        for i in np.atleast_1d(ix):
            self.setDriveOne(int(i), rate)

    def set_array(self, name: str, values):
        """Replace logGain / outScale / thrOffset / bias (per neuron) or edgeGain (per edge)."""
        key = {"logGain": "log_gain", "outScale": "out_scale", "thrOffset": "thr_offset",
               "bias": "bias", "edgeGain": "edge_gain"}.get(name, name)
        if hasattr(values, "data_ptr"):
            nat.check(self.L.fb_diff_set(self.h, _FIELDS[key], C.c_void_p(values.data_ptr())))
            return
        v = np.ascontiguousarray(values, np.float32)
        self.arrays[key] = v
        nat.check(self.L.fb_diff_set(self.h, _FIELDS[key], v.ctypes.data))

    def params(self, **over) -> nat.FbDiffParams:
        return make_params(dict(self.p, **over))

    def forward(self, steps: int, seed: int = 1, record: bool = True, **over):
        """Runs from reset; returns spikeCount f32[N] (src/lifdiff.js:219)."""
        if self._drive_dirty:
            self._create(self._tape_cap)
        sc = np.zeros(self.N, np.float32)
        self._last = dict(steps=steps, seed=seed, over=over)
        nat.check(self.L.fb_diff_forward(self.h, C.byref(self.params(**over)), int(steps), int(seed),
                                         1 if record else 0, sc.ctypes.data))
        self.spikeCount = sc
        return sc

    def tape(self):
        """(offsets i64[steps+1], idx, amp) of the recorded forward."""
        steps = self._last["steps"]
        off = np.zeros(steps + 1, np.int64)
        n = C.c_int64()
        nat.check(self.L.fb_diff_tape(self.h, off.ctypes.data, None, None, 0, C.byref(n)))
        idx = np.zeros(max(1, n.value), np.int32)
        amp = np.zeros(max(1, n.value), np.float32)
        nat.check(self.L.fb_diff_tape(self.h, off.ctypes.data, idx.ctypes.data, amp.ctypes.data, n.value, C.byref(n)))
        return off, idx[: n.value], amp[: n.value]

    def raster(self, readout, out=None):
        """Dense f32[steps][len(readout)] raster of the recorded forward (host, or into a torch
        CUDA tensor `out`)."""
        ro = np.ascontiguousarray(readout, np.int32)
        if out is None:
            out = np.zeros((self._last["steps"], ro.shape[0]), np.float32)
            nat.check(self.L.fb_diff_raster(self.h, ro.shape[0], ro.ctypes.data, out.ctypes.data))
            return out
        nat.check(self.L.fb_diff_raster(self.h, ro.shape[0], ro.ctypes.data, C.c_void_p(out.data_ptr())))
        return out

    def backward(self, dLdSpike, truncate: int = 0, lossFrom: int = 0, readout=None, edge: bool = True):
        """src/lifdiff.js:494: dLdSpike f32[N] (every scored step), or f32[steps][len(readout)]
        with readout indices. Returns {params, logGain, clamped, edge, bias, outScale}."""
        g = nat.FbDiffGrads()
        lg = np.zeros(self.N, np.float32)
        ge = np.zeros(self.E, np.float64) if edge else None
        gb = np.zeros(self.N, np.float64)
        go = np.zeros(self.N, np.float64)
        g.log_gain, g.bias, g.out_scale = lg.ctypes.data, gb.ctypes.data, go.ctypes.data
        g.edge = None if ge is None else ge.ctypes.data
        if hasattr(dLdSpike, "data_ptr"):
            dptr = C.c_void_p(dLdSpike.data_ptr())
        else:
            dl = np.ascontiguousarray(dLdSpike, np.float32)
            dptr = dl.ctypes.data
        ro = None if readout is None else np.ascontiguousarray(readout, np.int32)
        nat.check(self.L.fb_diff_backward(self.h, dptr, 0 if ro is None else ro.shape[0],
                                          None if ro is None else ro.ctypes.data, int(truncate),
                                          int(lossFrom), C.byref(g)))
        return dict(params=dict(zip(DIFF_PARAMS, list(g.params))), logGain=lg,
                    clamped=dict(params=g.clamped_params, logGain=g.clamped_log_gain),
                    edge=ge, bias=gb, outScale=go, truncate=truncate)
