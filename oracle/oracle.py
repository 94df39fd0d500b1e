"""ORACLE -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module, and only as the checker (or the timed CPU port); no product path calls it.

It restates the reference's host glue around the brain step -- ``LIFWasm`` in src/lifwasm.js --
over two interchangeable C backends with the same ``ob_*`` interface:

* ``"port"``: oracle/lifsim.c, a C restatement of src/wasm/lif.c:29-80;
* ``"ref"``: the reference src/wasm/lif.c itself, compiled natively from the reference tree by
  oracle/Makefile into oracle/_ref/ (present only where the reference tree is).

The port is pinned bit-for-bit against the reference build on the golden cases in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liblifsim.so")
REF_LIB = os.path.join(HERE, "_ref", "libreflif.so")

# src/lif.js:6-15 (DEFAULTS) -- the parameter set LIFWasm merges caller params over.
DEFAULTS = dict(
    dt=0.5, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
    wSyn=0.275, noise=0.0, traceTau=30.0, adaptInc=2.0, adaptTau=100.0, depU=0.2, depTau=200.0,
    minSyn=1, preInh=0.0, coba=False, eExc=0.0, eInh=-70.0, inhGain=1.0, bgRate=0.0, bgAmp=0.0,
)


class OHdr(C.Structure):
    """Scalar header of oracle/lifsim.c (same layout in oracle/ref_harness.c)."""

    _fields_ = [
        ("N", C.c_int32), ("nslots", C.c_int32), ("head", C.c_int32), ("coba", C.c_int32),
        ("c", C.c_float * 17), ("rng", C.c_uint32),
        ("nDriven", C.c_int32), ("nFired", C.c_int32), ("lastSlot", C.c_int32),
        ("bgEvents", C.c_float), ("bgAmp", C.c_float), ("bgAcc", C.c_float), ("preInh", C.c_float),
    ]


def build(ref: bool | None = None) -> None:
    """Compile the oracle libraries; with ref None the Makefile also builds the reference kernel
    when it finds the reference tree (FLYBRAIN_REFERENCE, else the Makefile's REF)."""
    cmd = ["make", "-s", "-C", HERE]
    root = os.environ.get("FLYBRAIN_REFERENCE")
    if root:
        cmd.append(f"REF={root}")
    targets = ["all"] if ref is None else (["port", "ref"] if ref else ["port"])
    subprocess.run(cmd + targets, check=True)


def have_reference_build() -> bool:
    """Whether the reference kernel was compiled here (the live-reference tests need it)."""
    return os.path.exists(REF_LIB)


_libs: dict[str, C.CDLL] = {}


def lib(backend: str = "port") -> C.CDLL:
    if backend in _libs:
        return _libs[backend]
    path = PORT_LIB if backend == "port" else REF_LIB
    if not os.path.exists(path):
        build(ref=(backend == "ref"))
    L = C.CDLL(path)
    P = C.c_void_p
    L.ob_create.restype = P
    L.ob_create.argtypes = [C.POINTER(OHdr)] + [P] * 18
    L.ob_set.argtypes = [P, C.POINTER(OHdr)]
    L.ob_get.argtypes = [P, C.POINTER(OHdr)]
    L.ob_destroy.argtypes = [P]
    L.ob_run.restype = C.c_int32
    L.ob_run.argtypes = [P, C.c_int32, P, P, C.c_int64, C.POINTER(C.c_int64)]
    L.ob_run_many.restype = C.c_int64
    L.ob_run_many.argtypes = [P, C.c_int32, P, C.c_int32]
    L.ob_threads.restype = C.c_int32
    _libs[backend] = L
    return L


def header_constants(p: dict) -> np.ndarray:
    """The 17 f32 header constants, each computed in f64 and rounded once to f32.

    Restates LIFWasm._writeHeader, src/lifwasm.js:59-61, in the header's order.
    """
    vals = [
        p["dt"], p["vRest"], p["vThresh"], p["vReset"], p["tRef"], p["adaptInc"], p["depU"],
        math.exp(-p["dt"] / p["tauSyn"]), math.exp(-p["dt"] / p["traceTau"]),
        math.exp(-p["dt"] / p["adaptTau"]), p["dt"] / p["depTau"], p["dt"] / p["tauM"],
        p["dt"] / 1000, p["eExc"], p["eInh"], 1 / (p["eExc"] - p["vRest"]),
        1 / (p["vRest"] - p["eInh"]),
    ]
    return np.array(vals, dtype=np.float64).astype(np.float32)


def n_slots(p: dict) -> int:
    """Delay-ring depth, src/lifwasm.js:39: max(1, round(delay/dt)) + 1 (JS Math.round)."""
    return max(1, int(math.floor(p["delay"] / p["dt"] + 0.5))) + 1


def seed_state(seed: int) -> int:
    """Initial xorshift32 state, src/lifwasm.js:52: (seed * 2654435761) >>> 0 || 1. JavaScript
    forms the product in double (rounded once when it exceeds 2^53, i.e. for seeds of 2^21 and
    more) and >>> 0 takes that double modulo 2^32."""
    x = math.fmod(math.floor(float(seed) * 2654435761.0), 4294967296.0)
    if x < 0:
        x += 4294967296.0
    return int(x) or 1


def write_graph_f64(N, indptr, indices, counts, nt_sign, p, in_scale=None, sensory_mask=None,
                    out_scale=None, edge_gain=None):
    """Restatement of writeGraph, src/lifwasm.js:14-34, with explicit per-edge loops in float64.

    ``nt_sign`` is the per-neuron sign before wSyn (preSign, or the transmitter sign table).
    Returns (W f32[E], sign f32[N]); each value is computed in f64 in the reference's operand
    order and rounded once to f32. Loops are plain Python: use on small graphs only.
    """
    E = len(indices)
    W = np.zeros(E, dtype=np.float32)
    sign = np.zeros(N, dtype=np.float32)
    for j in range(N):
        s = float(nt_sign[j])
        sign[j] = np.float32(s * p["wSyn"])
        og = float(out_scale[j]) if out_scale is not None else 1.0
        ig = (p["inhGain"] if s < 0 else 1.0) * og
        for k in range(int(indptr[j]), int(indptr[j + 1])):
            q = int(indices[k])
            c = float(counts[k])
            keep = not (sensory_mask is not None and sensory_mask[q]) or (p["preInh"] > 0 and s < 0)
            if c >= p["minSyn"] and keep:
                val = c * (float(edge_gain[k]) if edge_gain is not None else 1.0)
                val = val * (float(in_scale[q]) if in_scale is not None else 1.0)
                W[k] = np.float32(val * ig)
    return W, sign


class OracleBrain:
    """CPU restatement of the LIFWasm brain object (src/lifwasm.js:36-87) over a C step kernel.

    Same surface as the reference: setDriveOne/setDrive/setBias/setThr/addG/pulse/reset/
    setBackground/step, the typed-array fields, and the insertion-ordered driven set that fixes
    the RNG draw order (src/lifwasm.js:70-71).
    """

    def __init__(self, N, indptr, indices, W, sign, params=None, seed=1, backend="port"):
        self.L = lib(backend)
        self.N = int(N)
        self.p = dict(DEFAULTS)
        self.p.update(params or {})
        p = self.p
        self.nslots = n_slots(p)
        self.indptr = np.ascontiguousarray(indptr, dtype=np.uint32)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32)
        self.W = np.ascontiguousarray(W, dtype=np.float32)
        self.sign = np.ascontiguousarray(sign, dtype=np.float32)
        f = lambda: np.zeros(self.N, dtype=np.float32)  # noqa: E731
        self.v, self.gE, self.gI, self.refr, self.trace = f(), f(), f(), f(), f()
        self.adapt, self.res, self.bias, self.thr, self.drive = f(), f(), f(), f(), f()
        self.spikeCount = np.zeros(self.N, dtype=np.uint32)
        self.ring = np.zeros(self.nslots * self.N, dtype=np.int32)
        self.ringCount = np.zeros(self.nslots, dtype=np.int32)
        self.drivenList = np.zeros(self.N, dtype=np.int32)
        self.drivenSet: dict[int, None] = {}  # dict keeps insertion order, like a JS Set
        self._dirty = True
        self.t = 0.0
        self.reset()
        self.hdr = OHdr()
        h = self.hdr
        h.N, h.nslots, h.head, h.coba = self.N, self.nslots, 0, 1 if p["coba"] else 0
        for k, v in enumerate(header_constants(p)):
            h.c[k] = float(v)
        h.rng = seed_state(seed)
        h.nDriven = h.nFired = h.lastSlot = 0
        h.bgEvents = float(np.float32(self.N * (p.get("bgRate") or 0) * p["dt"] / 1000))
        h.bgAmp = float(np.float32(p.get("bgAmp") or 0))
        h.bgAcc = 0.0
        h.preInh = float(np.float32(p.get("preInh") or 0))
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        self._h = self.L.ob_create(
            C.byref(h), ptr(self.v), ptr(self.gE), ptr(self.gI), ptr(self.refr), ptr(self.trace),
            ptr(self.adapt), ptr(self.res), ptr(self.bias), ptr(self.thr), ptr(self.drive),
            ptr(self.sign), ptr(self.spikeCount), ptr(self.indptr), ptr(self.indices), ptr(self.W),
            ptr(self.ring), ptr(self.ringCount), ptr(self.drivenList))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self.L.ob_destroy(h)
            self._h = None

    # -- header access ---------------------------------------------------------------------
    def _pull(self):
        self.L.ob_get(self._h, C.byref(self.hdr))
        return self.hdr

    def _push(self):
        self.L.ob_set(self._h, C.byref(self.hdr))

    @property
    def head(self):
        return self._pull().head

    @property
    def rng(self):
        return self._pull().rng

    # -- LIFWasm API (src/lifwasm.js:69-86) --------------------------------------------------
    def setBackground(self, rate_hz, amp_mv):
        self._pull()
        self.p["bgRate"], self.p["bgAmp"] = rate_hz, amp_mv
        self.hdr.bgEvents = float(np.float32(self.N * rate_hz * self.p["dt"] / 1000))
        self.hdr.bgAmp = float(np.float32(amp_mv))
        self._push()

    def _syncDriven(self):
        n = 0
        for i in self.drivenSet:
            self.drivenList[n] = i
            n += 1
        self._pull()
        self.hdr.nDriven = n
        self._push()
        self._dirty = False

    def setDriveOne(self, i, rate):
        i = int(i)
        self.drive[i] = rate
        if rate > 0:
            if i not in self.drivenSet:
                self.drivenSet[i] = None
                self._dirty = True
        elif i in self.drivenSet:
            del self.drivenSet[i]
            self._dirty = True

    def setDrive(self, ix, rate):
        for i in ix:
            self.setDriveOne(i, rate)

    def setBias(self, ix, mv):
        for i in ix:
            self.bias[int(i)] = mv

    def setThr(self, i, mv):
        self.thr[int(i)] = mv

    def addG(self, i, e, ii=0.0):
        """src/lifwasm.js:75. A Float32Array element plus a JS number: the sum is formed in f64
        and rounded once on the store."""
        i = int(i)
        self.gE[i] = np.float32(float(self.gE[i]) + float(e))
        self.gI[i] = np.float32(float(self.gI[i]) + float(ii or 0.0))

    def pulse(self, ix, mv):
        """src/lifwasm.js:76, with the same f64-then-round store as addG."""
        for i in ix:
            i = int(i)
            self.gE[i] = np.float32(float(self.gE[i]) + float(mv))

    def wake(self, *a):
        pass

    def reset(self):
        """src/lifwasm.js:78: state back to rest; head, RNG and background accumulator untouched."""
        self.v.fill(np.float32(self.p["vRest"]))
        for a in (self.gE, self.gI, self.refr, self.trace, self.adapt):
            a.fill(0)
        self.res.fill(1)
        self.spikeCount.fill(0)
        self.ringCount.fill(0)
        self.t = 0.0

    def step(self):
        """One step; returns the fired list (a copy of the ring slot written this step)."""
        if self._dirty:
            self._syncDriven()
        nf = self.L.ob_run(self._h, 1, None, None, 0, None)
        self.t += self.p["dt"]
        slot = self._pull().lastSlot
        return self.ring[slot * self.N: slot * self.N + nf].copy()

    def run(self, nsteps, raster=False):
        """nsteps steps in C. Returns per-step fired counts, and the concatenated raster if asked."""
        if self._dirty:
            self._syncDriven()
        nf = np.zeros(nsteps, dtype=np.int32)
        if raster:
            cap = C.c_int64(0)
            buf = np.zeros(1 << 16, dtype=np.int32)
            # two passes would replay the RNG; instead grow the buffer from a count-only copy
            h0 = OHdr.from_buffer_copy(self._pull())
            snap = self._snapshot()
            self.L.ob_run(self._h, nsteps, None, None, 0, C.byref(cap))
            self._restore(snap, h0)
            buf = np.zeros(max(1, cap.value), dtype=np.int32)
            n = C.c_int64(0)
            self.L.ob_run(self._h, nsteps, nf.ctypes.data_as(C.c_void_p),
                          buf.ctypes.data_as(C.c_void_p), cap.value, C.byref(n))
            self.t += nsteps * self.p["dt"]
            return nf, buf[: n.value]
        self.L.ob_run(self._h, nsteps, nf.ctypes.data_as(C.c_void_p), None, 0, None)
        self.t += nsteps * self.p["dt"]
        return nf

    _STATE = ("v", "gE", "gI", "refr", "trace", "adapt", "res", "spikeCount", "ring", "ringCount")

    def _snapshot(self):
        return {k: getattr(self, k).copy() for k in self._STATE}

    def _restore(self, snap, hdr):
        for k in self._STATE:
            getattr(self, k)[...] = snap[k]
        self.hdr = hdr
        self._push()

    @property
    def nAwake(self):
        return self.N


def run_many(brains, steps, nthreads: int = 0) -> int:
    """Advances independent oracle brains (graphs may be shared) by steps[k] steps each, in
    parallel over nthreads host threads (<= 0: all): ob_run_many, the CPU counterpart of a batched
    ensemble. Returns the total fired count."""
    if not brains:
        return 0
    L = brains[0].L
    for b in brains:
        if b._dirty:
            b._syncDriven()
    hs = (C.c_void_p * len(brains))(*[b._h for b in brains])
    st = np.ascontiguousarray(steps, dtype=np.int32)
    n = int(L.ob_run_many(hs, len(brains), st.ctypes.data_as(C.c_void_p), int(nthreads)))
    for b, k in zip(brains, st.tolist()):
        b.t += k * b.p["dt"]
    return n


def fv_run(model: dict, v, x, steps: int, backend: str = "port", nthreads: int = 0, kdt=None):
    """B flyvis instances (v, x: float32 [B][N]) advanced `steps` fv_steps in place by the oracle
    restatement (backend "port") or the reference's own fv_step (backend "ref",
    src/wasm/lif.c:86-93). kdt defaults to dt / max(tau, dt) rounded to f32 (src/flyvis.js:13)."""
    L = lib(backend)
    if not hasattr(L, "_fv_bound"):
        L.ob_fv_run.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
        L._fv_bound = True
    N = int(model["N"])
    if kdt is None:
        dt = float(model.get("dt") or 0.02)
        kdt = (dt / np.maximum(np.asarray(model["tau"], np.float64), dt)).astype(np.float32)
    arrs = [np.ascontiguousarray(model["bias"], np.float32), np.ascontiguousarray(kdt, np.float32),
            np.ascontiguousarray(model["indptr"], np.int32), np.ascontiguousarray(model["target"], np.int32),
            np.ascontiguousarray(model["weight"], np.float32)]
    assert v.dtype == np.float32 and v.flags.c_contiguous and x.dtype == np.float32 and x.flags.c_contiguous
    B = v.size // N
    L.ob_fv_run(N, *[a.ctypes.data for a in arrs], B, v.ctypes.data, np.ascontiguousarray(x).ctypes.data,
                int(steps), int(nthreads))
    return v
