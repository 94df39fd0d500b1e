"""The differentiable brain on the GB300 kernels: a drop-in for the reference's LIFDiff
(src/lifdiff.js:77-687) -- new LIFDiff(data, opts), setDrive/setDriveOne, forward(steps,
{seed, record, onEpoch, spikeTrain}) and backward(tape, dLdSpike, {truncate, lossFrom}) returning
{params, logGain, drive, clamped} -- plus per-edge, per-neuron-bias and outScale gradients, and a
torch.autograd.Function over per-edge gains, per-neuron biases and per-cell-type gains.

The reference's onEpoch callback is given as its result: driveAt[epoch][k], the drive of
driveIdx[k] from that epoch's first step, applied with setDriveOne in k order.
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
    precision="f64", driveSoft=False, exact32=False, driveEpoch=1,
)
_INT_PARAMS = ("coba", "soft", "checkpoint", "precision", "drive_soft", "exact32", "drive_epoch", "pad")
PRECISIONS = dict(f64=0, f32=1)

_ARRAYS_N = ("size_log", "in_scale", "log_gain", "out_scale", "thr_offset", "beta", "bias")
_MASKS = ("thr_mask", "bias_mask", "sensory")
_FIELDS = dict(log_gain=0, out_scale=1, thr_offset=2, bias=3, edge_gain=4, drive=5)


def make_params(p: dict) -> nat.FbDiffParams:
    q = nat.FbDiffParams()
    for k, _ in nat.FbDiffParams._fields_:
        if k in _INT_PARAMS:
            continue
        setattr(q, k, float(p[k]))
    q.coba, q.soft, q.checkpoint = int(bool(p["coba"])), int(bool(p["soft"])), int(p["checkpoint"])
    q.drive_soft, q.exact32 = int(bool(p["driveSoft"])), int(bool(p["exact32"]))
    q.drive_epoch = max(1, int(p["driveEpoch"] or 1))
    if p["precision"] not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, not {p['precision']!r}")
    q.precision = PRECISIONS[p["precision"]]
    return q


class _Desc:
    """Builds fb_diff_net records; the same array object given for the same field of several
    networks yields the same pointer, so the library uploads it once."""

    def __init__(self):
        self.keep = []
        self._cache = {}

    def arr(self, x, dt):
        if x is None:
            return None
        key = (id(x), np.dtype(dt).str)
        hit = self._cache.get(key)
        if hit is not None and hit[0] is x:
            return hit[1].ctypes.data
        a = np.ascontiguousarray(x, dt)
        self.keep += [a, x]
        self._cache[key] = (x, a)
        return a.ctypes.data

    def net(self, n: "DiffNet", out: nat.FbDiffNet):
        out.N, out.E = n.N, n.E
        out.indptr, out.indices = self.arr(n.indptr, np.uint32), self.arr(n.indices, np.uint32)
        out.counts, out.sign = self.arr(n.counts, np.float32), self.arr(n.sign, np.float32)
        for k in _ARRAYS_N + ("edge_gain",):
            setattr(out, k, self.arr(n.arrays[k], np.float32))
        for k in _MASKS:
            setattr(out, k, self.arr(n.arrays[k], np.uint8))
        driven = np.array(list(n.drivenSet), np.int32)
        out.nDriven = int(driven.shape[0])
        out.drive = self.arr(n.drive.copy(), np.float32)
        out.driven = self.arr(driven if driven.shape[0] else np.zeros(1, np.int32), np.int32)
        if n.driveIdx is not None:
            out.nDriveIdx = int(n.driveIdx.shape[0])
            out.drive_idx = self.arr(n.driveIdx, np.int32)


def _epochs(steps, p):
    ep = max(1, int(p["driveEpoch"] or 1))
    return (int(steps) + ep - 1) // ep


class _Inputs:
    """An fb_diff_inputs record: a drive schedule f32[epochs][nDriveIdx] and a spike train (one
    index list, or None, per step) as CSR offsets and indices."""

    def __init__(self, n, steps, p, driveAt=None, spikeTrain=None):
        self.rec = nat.FbDiffInputs()
        self.keep = []
        if driveAt is not None:
            if n.driveIdx is None:
                raise ValueError("driveAt needs the network's driveIdx")
            a = np.ascontiguousarray(driveAt, np.float32)
            want = (_epochs(steps, p), n.driveIdx.shape[0])
            if a.size != want[0] * want[1]:
                raise ValueError(f"driveAt must hold {want[0]} x {want[1]} values, not {a.shape}")
            self.keep.append(a)
            self.rec.drive_at = a.ctypes.data
        if spikeTrain is not None:
            if len(spikeTrain) < steps:
                raise ValueError(f"spikeTrain has {len(spikeTrain)} steps, the forward {steps}")
            lens = [0 if spikeTrain[t] is None else len(spikeTrain[t]) for t in range(steps)]
            off = np.zeros(steps + 1, np.int64)
            np.cumsum(lens, out=off[1:])
            idx = np.zeros(max(1, int(off[-1])), np.int32)
            for t in range(steps):
                if lens[t]:
                    idx[off[t]:off[t + 1]] = np.asarray(spikeTrain[t], np.int32)
            self.keep += [off, idx]
            self.rec.train_off, self.rec.train_idx = off.ctypes.data, idx.ctypes.data


def _grads(N, E, edge=True, device=None, drive_shape=None):
    """An FbDiffGrads with its output arrays (numpy, or torch tensors on `device`); drive_shape
    (epochs, nDriveIdx) adds the drive gradient."""
    g = nat.FbDiffGrads()
    if device is None:
        lg, gb, go = np.zeros(N, np.float32), np.zeros(N, np.float64), np.zeros(N, np.float64)
        ge = np.zeros(E, np.float64) if edge else None
        gd = None if drive_shape is None else np.zeros(drive_shape, np.float32)
        ptr = lambda a: a.ctypes.data  # noqa: E731
    else:
        import torch
        lg = torch.zeros(N, dtype=torch.float32, device=device)
        gb, go = (torch.zeros(N, dtype=torch.float64, device=device) for _ in range(2))
        ge = torch.zeros(E, dtype=torch.float64, device=device) if edge else None
        gd = None if drive_shape is None else torch.zeros(drive_shape, dtype=torch.float32, device=device)
        ptr = lambda a: a.data_ptr()  # noqa: E731
    g.log_gain, g.bias, g.out_scale = ptr(lg), ptr(gb), ptr(go)
    g.edge = None if ge is None else ptr(ge)
    g.drive = None if gd is None else ptr(gd)
    return g, dict(logGain=lg, edge=ge, bias=gb, outScale=go, drive=gd)


def _grad_dict(g, arrays, truncate):
    return dict(params=dict(zip(DIFF_PARAMS, list(g.params))),
                clamped=dict(params=g.clamped_params, logGain=g.clamped_log_gain, drive=g.clamped_drive),
                truncate=truncate, **arrays)


def _dl_ptr(x):
    if x is None:
        return None, None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr()).value, x
    a = np.ascontiguousarray(x, np.float32)
    return a.ctypes.data, a


class DiffNet:
    """LIFDiff on the device. data: {N, indptr, indices, weights (raw counts), nt} as the
    reference takes it (or sign= for preSign); opts: model parameters and per-neuron structure
    (sizeLog, thrMask, biasMask, logGain, outScale, thrOffset, sensoryMask, edgeGain, inScale,
    surrogateBeta as an array, bias, driveIdx)."""

    def __init__(self, data: dict, opts: dict | None = None, tape_cap: int = 0, _defer: bool = False):
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
        di = opts.get("driveIdx")
        self.driveIdx = None if di is None else np.ascontiguousarray(di, np.int32)
        self.h = None
        self._tape_cap = tape_cap
        if not _defer:
            self._create(tape_cap)

    def _create(self, tape_cap):
        desc = _Desc()
        net = nat.FbDiffNet()
        desc.net(self, net)
        h = C.c_void_p()
        nat.check(self.L.fb_diff_create(C.byref(net), int(tape_cap), C.byref(h)))
        if self.h:
            self.L.fb_diff_destroy(self.h)
        self.h = h
        self._tape_cap = tape_cap
        self._drive_dirty = False
        # arrays set from device tensors are not in the host record the handle is built from:
        # a rebuilt handle (after a drive change) gets them again
        for key, t in getattr(self, "_dev_arrays", {}).items():
            nat.check(self.L.fb_diff_set(self.h, _FIELDS[key], C.c_void_p(t.data_ptr())))

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
        if self._drive_dirty and self.h is not None:
            self._create(self._tape_cap)  # a pending drive change rebuilds the handle: first, not after
        if not hasattr(self, "_dev_arrays"):
            self._dev_arrays = {}
        if hasattr(values, "data_ptr"):
            t = values.detach().contiguous().clone()
            self._dev_arrays[key] = t
            nat.check(self.L.fb_diff_set(self.h, _FIELDS[key], C.c_void_p(t.data_ptr())))
            return
        self._dev_arrays.pop(key, None)
        v = np.ascontiguousarray(values, np.float32)
        self.arrays[key] = v
        nat.check(self.L.fb_diff_set(self.h, _FIELDS[key], v.ctypes.data))

    def params(self, **over) -> nat.FbDiffParams:
        return make_params(dict(self.p, **over))

    def forward(self, steps: int, seed: int = 1, record: bool = True, driveAt=None, spikeTrain=None, **over):
        """Runs from reset; returns spikeCount f32[N] (src/lifdiff.js:219). driveAt: the drive
        schedule f32[epochs][len(driveIdx)]; spikeTrain: per step a list of neurons to force."""
        if self._drive_dirty:
            self._create(self._tape_cap)
        sc = np.zeros(self.N, np.float32)
        p = dict(self.p, **over)
        self._last = dict(steps=steps, seed=seed, over=over, p=p)
        ins = _Inputs(self, steps, p, driveAt, spikeTrain)
        nat.check(self.L.fb_diff_forward_ex(self.h, C.byref(make_params(p)), int(steps), int(seed),
                                            1 if record else 0, sc.ctypes.data, C.byref(ins.rec)))
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

    def backward(self, dLdSpike, truncate: int = 0, lossFrom: int = 0, readout=None, edge: bool = True,
                 device=None):
        """src/lifdiff.js:494: dLdSpike f32[N] (every scored step), or f32[steps][len(readout)]
        with readout indices. Returns {params, logGain, drive, clamped, edge, bias, outScale}
        (numpy, or torch tensors on `device`); drive is f32[epochs][len(driveIdx)] or None."""
        ds = None if self.driveIdx is None else (_epochs(self._last["steps"], self._last["p"]), self.driveIdx.shape[0])
        g, arrays = _grads(self.N, self.E, edge, device, ds)
        dptr, _keep = _dl_ptr(dLdSpike)
        ro = None if readout is None else np.ascontiguousarray(readout, np.int32)
        nat.check(self.L.fb_diff_backward(self.h, dptr, 0 if ro is None else ro.shape[0],
                                          None if ro is None else ro.ctypes.data, int(truncate),
                                          int(lossFrom), C.byref(g)))
        return _grad_dict(g, arrays, truncate)


class DiffBatch:
    """B independent differentiable brains advanced together, every launch covering all members
    and each forward or backward pass replayed as one captured CUDA graph
    (fb_diff_batch_*): each member is a DiffNet built with DiffNet(..., _defer=True) (its graph,
    per-neuron arrays and driven set); the model parameters are the batch's. Arrays that are the
    same object in several members are uploaded once and shared."""

    def __init__(self, members, params: dict | None = None, tape_cap: int = 0):
        self.L = nat.load()
        self.members = list(members)
        self.B = len(self.members)
        self.p = dict(DIFF_DEFAULTS, **(params or {}))
        self.N = [m.N for m in self.members]
        self.E = [m.E for m in self.members]
        desc = _Desc()
        nets = (nat.FbDiffNet * self.B)()
        for b, m in enumerate(self.members):
            desc.net(m, nets[b])
        h = C.c_void_p()
        nat.check(self.L.fb_diff_batch_create(nets, self.B, int(tape_cap), C.byref(h)))
        self.h = h
        self._steps = [0] * self.B
        self._p = self.p
        self.tuning = dict(neuron_blocks=0, arrival_blocks=0, step_launches=False)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.fb_diff_batch_destroy(h)
            self.h = None

    def set_tuning(self, neuron_blocks: int = 0, arrival_blocks: int = 0, step_launches: bool | None = None):
        """Launch shape of the per-step kernels (fb_diff_batch_set_tuning); 0 = default.
        step_launches: True launches every step's kernels from the host, False replays each pass
        as a captured CUDA graph (the default); None keeps the current choice."""
        sl = self.tuning.get("step_launches", False) if step_launches is None else bool(step_launches)
        t = nat.FbDiffTuning(int(neuron_blocks), int(arrival_blocks), int(sl))
        nat.check(self.L.fb_diff_batch_set_tuning(self.h, C.byref(t)))
        self.tuning = dict(neuron_blocks=int(neuron_blocks), arrival_blocks=int(arrival_blocks), step_launches=sl)

    def set_array(self, inst: int, name: str, values):
        key = {"logGain": "log_gain", "outScale": "out_scale", "thrOffset": "thr_offset",
               "bias": "bias", "edgeGain": "edge_gain", "drive": "drive"}.get(name, name)
        if hasattr(values, "data_ptr"):
            ptr = C.c_void_p(values.data_ptr())
        else:
            v = np.ascontiguousarray(values, np.float32)
            ptr = v.ctypes.data
        nat.check(self.L.fb_diff_batch_set(self.h, int(inst), _FIELDS[key], ptr))

    def forward(self, steps, seeds=1, record: bool = True, counts: bool = True, driveAt=None,
                spikeTrain=None, **over):
        """Every member from reset for steps[b] steps with seeds[b]; returns the members' spike
        counts (or None with counts=False). driveAt / spikeTrain: per member (lists, entries may
        be None) as DiffNet.forward takes them."""
        st = np.broadcast_to(np.asarray(steps, np.int32), (self.B,)).copy()
        sd = np.broadcast_to(np.asarray(seeds, np.uint32), (self.B,)).copy()
        sc = np.zeros(sum(self.N), np.float32) if counts else None
        p = dict(self.p, **over)
        ins = [_Inputs(m, int(st[b]), p, None if driveAt is None else driveAt[b],
                       None if spikeTrain is None else spikeTrain[b]) for b, m in enumerate(self.members)]
        recs = (nat.FbDiffInputs * self.B)(*[x.rec for x in ins])
        nat.check(self.L.fb_diff_batch_forward_ex(self.h, C.byref(make_params(p)), st.ctypes.data,
                                                  sd.ctypes.data, 1 if record else 0,
                                                  None if sc is None else sc.ctypes.data, recs))
        self._steps = st.tolist()
        self._p = p
        if sc is None:
            return None
        return np.split(sc, np.cumsum(self.N)[:-1])

    def tape(self, inst: int):
        steps = self._steps[inst]
        off = np.zeros(steps + 1, np.int64)
        n = C.c_int64()
        nat.check(self.L.fb_diff_batch_tape(self.h, int(inst), off.ctypes.data, None, None, 0, C.byref(n)))
        idx = np.zeros(max(1, n.value), np.int32)
        amp = np.zeros(max(1, n.value), np.float32)
        nat.check(self.L.fb_diff_batch_tape(self.h, int(inst), off.ctypes.data, idx.ctypes.data, amp.ctypes.data,
                                            n.value, C.byref(n)))
        return off, idx[: n.value], amp[: n.value]

    def raster(self, inst: int, readout, out=None):
        ro = np.ascontiguousarray(readout, np.int32)
        if out is None:
            out = np.zeros((self._steps[inst], ro.shape[0]), np.float32)
            nat.check(self.L.fb_diff_batch_raster(self.h, int(inst), ro.shape[0], ro.ctypes.data, out.ctypes.data))
            return out
        nat.check(self.L.fb_diff_batch_raster(self.h, int(inst), ro.shape[0], ro.ctypes.data,
                                              C.c_void_p(out.data_ptr())))
        return out

    def rasters(self, readouts, outs):
        """Every member's readout raster at once: member k's (steps_k x len(readouts[k]))
        amplitudes into the torch CUDA tensor outs[k] (fb_diff_batch_rasters)."""
        ros = [np.ascontiguousarray(r, np.int32) for r in readouts]
        nro = np.array([r.shape[0] for r in ros], np.int32)
        rp = (C.c_void_p * self.B)(*[r.ctypes.data for r in ros])
        op = (C.c_void_p * self.B)(*[o.data_ptr() for o in outs])
        nat.check(self.L.fb_diff_batch_rasters(self.h, nat.ptr(nro), rp, op))
        return outs

    def backward(self, dLs, readouts=None, truncate: int = 0, lossFrom: int = 0, edge: bool = True, device=None):
        """Per member: dLs[b] as DiffNet.backward's dLdSpike (readouts[b] its readout set or None).
        Returns one gradient dict per member."""
        B = self.B
        ptrs = (C.c_void_p * B)()
        nro = np.zeros(B, np.int32)
        ros = (C.c_void_p * B)()
        keep = []
        for b in range(B):
            ptrs[b], k = _dl_ptr(dLs[b])
            keep.append(k)
            ro = None if readouts is None or readouts[b] is None else np.ascontiguousarray(readouts[b], np.int32)
            if ro is not None:
                keep.append(ro)
                nro[b] = ro.shape[0]
                ros[b] = ro.ctypes.data
        gs = (nat.FbDiffGrads * B)()
        arrays = []
        for b in range(B):
            m = self.members[b]
            ds = None if m.driveIdx is None else (_epochs(self._steps[b], self._p), m.driveIdx.shape[0])
            g, a = _grads(self.N[b], self.E[b], edge, device, ds)
            gs[b] = g
            arrays.append(a)
        nat.check(self.L.fb_diff_batch_backward(self.h, ptrs, nro.ctypes.data, ros, int(truncate), int(lossFrom), gs))
        return [_grad_dict(gs[b], arrays[b], truncate) for b in range(B)]

    def edge_sum(self, insts=None, out=None):
        """Per-edge gradients of the listed members (all by default) summed in list order."""
        ii = np.ascontiguousarray(range(self.B) if insts is None else insts, np.int32)
        E = self.E[int(ii[0])]
        if out is None:
            out = np.zeros(E, np.float64)
            nat.check(self.L.fb_diff_batch_edge_sum(self.h, ii.shape[0], ii.ctypes.data, out.ctypes.data))
            return out
        nat.check(self.L.fb_diff_batch_edge_sum(self.h, ii.shape[0], ii.ctypes.data, C.c_void_p(out.data_ptr())))
        return out
