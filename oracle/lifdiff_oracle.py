"""ORACLE -- test infrastructure only (the checker for the adjoint; no product path calls it).

ctypes wrapper of oracle/lifdiff.c, the C restatement of the reference's LIFDiff
(src/lifdiff.js:219-686). Parity: pinned by central finite differences (scripts/grad_check.mjs's
tolerance), not by the reference's own outputs (Node, which runs it, is absent here).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import oracle as _o

LIB = os.path.join(_o.HERE, "_build", "liblifdiff.so")

# LIFDiff defaults, src/lifdiff.js:85-110
DIFF_DEFAULTS = dict(
    dt=0.5, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
    wSyn=0.3, adaptInc=0.0, adaptTau=100.0, depU=0.0, depTau=200.0, minSyn=1.0, coba=True,
    eExc=0.0, eInh=-70.0, inhGain=1.0, sizeAlpha=0.0, maxSizeScale=20.0, boostCap=1.0,
    kcThreshold=0.0, laminaBias=0.0, surrogateBeta=2.0, adjClip=0.0, soft=False,
    driveSoft=False, exact32=False, driveEpoch=1,
)
DIFF_PARAMS = ["wSyn", "sizeAlpha", "inhGain", "eInh", "vThresh", "kcThreshold", "laminaBias",
               "adaptInc", "depU"]  # src/lifdiff.js:75


class LdParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "wSyn", "adaptInc",
        "adaptTau", "depU", "depTau", "minSyn", "eExc", "eInh", "inhGain", "sizeAlpha",
        "maxSizeScale", "boostCap", "kcThreshold", "laminaBias", "surrogateBeta", "adjClip")] + [
        (k, C.c_int32) for k in ("coba", "soft", "checkpoint", "truncate", "lossFrom", "steps")] + [
        ("seed", C.c_uint32), ("nDriven", C.c_int32), ("driveSoft", C.c_int32), ("exact32", C.c_int32),
        ("driveEpoch", C.c_int32), ("nDriveIdx", C.c_int32)]


class LdGraph(C.Structure):
    _fields_ = [("N", C.c_int32), ("E", C.c_int64)] + [(k, C.c_void_p) for k in (
        "indptr", "indices", "counts", "edgeGain", "sign", "sizeLog", "inScaleSrc", "logGain",
        "outScale", "thrOffset", "beta", "thrMask", "biasMask", "sensory", "drive", "driven", "driveIdx",
        "driveAt", "trainOff", "trainIdx")]


class LdGrads(C.Structure):
    _fields_ = [("params", C.c_double * 9), ("clamped_params", C.c_int32),
                ("clamped_logGain", C.c_int32), ("logGain", C.c_void_p), ("gEdge", C.c_void_p),
                ("gBias", C.c_void_p), ("gOut", C.c_void_p), ("gDrive", C.c_void_p),
                ("clamped_drive", C.c_int32), ("pad", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            _o.build(ref=False)
        L = C.CDLL(LIB)
        L.ld_forward.restype = C.c_int64
        L.ld_forward.argtypes = [C.POINTER(LdParams), C.POINTER(LdGraph)] + [C.c_void_p] * 5 + [
            C.c_int64, C.c_void_p, C.c_void_p]
        L.ld_backward.restype = C.c_int32
        L.ld_backward.argtypes = [C.POINTER(LdParams), C.POINTER(LdGraph)] + [C.c_void_p] * 7 + [
            C.c_int32, C.POINTER(LdGrads)]
        _lib = L
    return _lib


def _p(a, dt=None):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=dt) if dt is not None else np.ascontiguousarray(a)


class DiffProblem:
    """A LIFDiff network: graph (raw counts), per-neuron structure, drive, parameters."""

    def __init__(self, N, indptr, indices, counts, sign, params=None, sizeLog=None, logGain=None,
                 outScale=None, thrOffset=None, thrMask=None, biasMask=None, sensory=None,
                 edgeGain=None, inScale=None, beta=None, driven=None, drive_hz=None, driveIdx=None):
        self.N = int(N)
        self.indptr = _p(indptr, np.uint32)
        self.indices = _p(indices, np.uint32)
        self.counts = _p(counts, np.float32)
        self.E = int(self.indices.shape[0])
        self.sign = _p(sign, np.float32)
        self.p = dict(DIFF_DEFAULTS, **(params or {}))
        z = lambda: np.zeros(self.N, np.float32)  # noqa: E731
        self.sizeLog = _p(sizeLog, np.float32) if sizeLog is not None else z()
        self.logGain = _p(logGain, np.float32) if logGain is not None else z()
        self.thrOffset = _p(thrOffset, np.float32) if thrOffset is not None else z()
        self.outScale = _p(outScale, np.float32)
        self.thrMask = _p(thrMask, np.uint8)
        self.biasMask = _p(biasMask, np.uint8)
        self.sensory = _p(sensory, np.uint8)
        self.edgeGain = _p(edgeGain, np.float32)
        self.inScale = _p(inScale, np.float32)
        self.beta = _p(beta, np.float32)
        self.driven = _p(driven if driven is not None else np.zeros(0), np.int32)
        self.drive = z()
        if driven is not None:
            self.drive[self.driven] = np.asarray(drive_hz, np.float64).astype(np.float32)
        self.driveIdx = _p(driveIdx, np.int32)

    def _structs(self, steps, seed, checkpoint, truncate=0, lossFrom=0, driveAt=None, spikeTrain=None, **over):
        p = dict(self.p, **over)
        P = LdParams()
        for k in ("dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "wSyn",
                  "adaptInc", "adaptTau", "depU", "depTau", "minSyn", "eExc", "eInh", "inhGain",
                  "sizeAlpha", "maxSizeScale", "boostCap", "kcThreshold", "laminaBias",
                  "surrogateBeta", "adjClip"):
            setattr(P, k, float(p[k]))
        P.coba, P.soft = int(bool(p["coba"])), int(bool(p["soft"]))
        P.checkpoint, P.truncate, P.lossFrom, P.steps = int(checkpoint), int(truncate), int(lossFrom), int(steps)
        P.seed, P.nDriven = int(seed), int(self.driven.shape[0])
        P.driveSoft, P.exact32 = int(bool(p["driveSoft"])), int(bool(p["exact32"]))
        P.driveEpoch = int(p["driveEpoch"])
        P.nDriveIdx = 0 if self.driveIdx is None else int(self.driveIdx.shape[0])
        G = LdGraph()
        G.N, G.E = self.N, self.E
        keep = dict(logGain=over.get("logGainArr", self.logGain))
        for k in ("indptr", "indices", "counts", "edgeGain", "sign", "sizeLog", "outScale",
                  "thrOffset", "beta", "thrMask", "biasMask", "sensory", "drive", "driven"):
            a = getattr(self, k)
            setattr(G, k, None if a is None else a.ctypes.data)
        G.inScaleSrc = None if self.inScale is None else self.inScale.ctypes.data
        lg = _p(keep["logGain"], np.float32)
        G.logGain = lg.ctypes.data
        extra = [lg]
        G.driveIdx = None if self.driveIdx is None else self.driveIdx.ctypes.data
        if driveAt is not None:
            da = _p(driveAt, np.float32)
            extra.append(da)
            G.driveAt = da.ctypes.data
        if spikeTrain is not None:  # list of index arrays, one per step
            lists = [[] if x is None else x for x in spikeTrain[:steps]]
            off = np.zeros(steps + 1, np.int64)
            off[1:] = np.cumsum([len(x) for x in lists] + [0] * max(0, steps - len(lists)))
            idx = np.concatenate([np.asarray(x, np.int32).reshape(-1) for x in lists] + [np.zeros(1, np.int32)])
            extra += [off, idx]
            G.trainOff, G.trainIdx = off.ctypes.data, idx.ctypes.data
        return P, G, extra

    def forward(self, steps, seed=1, checkpoint=16, driveAt=None, spikeTrain=None, **over):
        """(spikeCount f32[N], tape) of a forward pass from reset (src/lifdiff.js:219). driveAt:
        [epochs][len(driveIdx)] drive schedule; spikeTrain: per step, the neurons forced then."""
        P, G, keep = self._structs(steps, seed, checkpoint, driveAt=driveAt, spikeTrain=spikeTrain, **over)
        cap = max(1024, steps * self.N)
        idx = np.zeros(cap, np.int32)
        amp = np.zeros(cap, np.float32)
        off = np.zeros(steps + 1, np.int64)
        forced = np.zeros(steps, np.int32)
        nck = (steps + checkpoint - 1) // checkpoint
        ck = np.zeros(max(1, nck) * 6 * self.N, np.float32)
        cks = np.zeros(max(1, nck), np.uint32)
        sc = np.zeros(self.N, np.float32)
        n = lib().ld_forward(C.byref(P), C.byref(G), sc.ctypes.data, idx.ctypes.data, amp.ctypes.data,
                             off.ctypes.data, forced.ctypes.data, cap, ck.ctypes.data, cks.ctypes.data)
        if n < 0:
            raise RuntimeError("tape capacity exceeded")
        tape = dict(idx=idx[:n], amp=amp[:n], off=off, forced=forced, ckpt=ck, ckptSeed=cks,
                    steps=steps, seed=seed, checkpoint=checkpoint, over=over, keep=keep,
                    driveAt=driveAt, spikeTrain=spikeTrain)
        return sc, tape

    def backward(self, tape, dL, truncate=0, lossFrom=0, edge=True):
        """Gradients of the reverse sweep (src/lifdiff.js:494-686) over a tape of forward()."""
        steps, K = tape["steps"], tape["checkpoint"]
        P, G, keep = self._structs(steps, tape["seed"], K, truncate=truncate, lossFrom=lossFrom,
                                   driveAt=tape["driveAt"], spikeTrain=tape["spikeTrain"], **tape["over"])
        dL = np.ascontiguousarray(dL, np.float32)
        per = 1 if dL.ndim == 2 else 0
        g = LdGrads()
        logGain = np.zeros(self.N, np.float32)
        gEdge = np.zeros(self.E, np.float64) if edge else None
        gBias = np.zeros(self.N, np.float64)
        gOut = np.zeros(self.N, np.float64)
        g.logGain = logGain.ctypes.data
        g.gEdge = None if gEdge is None else gEdge.ctypes.data
        g.gBias, g.gOut = gBias.ctypes.data, gOut.ctypes.data
        gDrive = None
        if tape["driveAt"] is not None and self.driveIdx is not None:
            ep = max(1, int(dict(self.p, **tape["over"])["driveEpoch"]))
            gDrive = np.zeros(((steps + ep - 1) // ep, self.driveIdx.shape[0]), np.float32)
            g.gDrive = gDrive.ctypes.data
        idx = np.ascontiguousarray(tape["idx"]) if tape["idx"].shape[0] else np.zeros(1, np.int32)
        amp = np.ascontiguousarray(tape["amp"]) if tape["amp"].shape[0] else np.zeros(1, np.float32)
        rc = lib().ld_backward(C.byref(P), C.byref(G), idx.ctypes.data, amp.ctypes.data,
                               tape["off"].ctypes.data, tape["forced"].ctypes.data,
                               tape["ckpt"].ctypes.data, tape["ckptSeed"].ctypes.data, dL.ctypes.data,
                               per, C.byref(g))
        if rc:
            raise RuntimeError("ld_backward failed")
        return dict(params=dict(zip(DIFF_PARAMS, list(g.params))), logGain=logGain, gEdge=gEdge,
                    gBias=gBias, gOut=gOut, drive=gDrive,
                    clamped=(g.clamped_params, g.clamped_logGain, g.clamped_drive))
