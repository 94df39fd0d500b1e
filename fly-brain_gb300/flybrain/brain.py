"""The reference's brain-model API on the GB300 step kernel.

``LIFCuda`` is a drop-in for ``LIFWasm`` (src/lifwasm.js:36-87): the same constructor arguments
(a compiled graph, params merged over DEFAULTS, a seed), the same methods
(step/setDriveOne/setDrive/setBias/setThr/addG/pulse/reset/setBackground/wake) and the same
readable fields (v, gE, gI, refr, trace, adapt, res, bias, thr, drive, spikeCount, drivenSet, t,
N, p, nAwake). Fields are read through from the device on access.

``BrainBatch`` is many such brains advanced by one persistent launch (the batched ensemble).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as nat
from .synth import Graph

# src/lif.js:6-15
DEFAULTS = dict(
    dt=0.5, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
    wSyn=0.275, noise=0.0, traceTau=30.0, adaptInc=2.0, adaptTau=100.0, depU=0.2, depTau=200.0,
    minSyn=1, preInh=0.0, coba=False, eExc=0.0, eInh=-70.0, inhGain=1.0, bgRate=0.0, bgAmp=0.0,
)


def make_params(p: dict) -> nat.FbParams:
    q = nat.FbParams()
    for k in ("dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "traceTau",
              "adaptInc", "adaptTau", "depU", "depTau", "eExc", "eInh", "bgRate", "bgAmp", "preInh"):
        setattr(q, k, float(p.get(k) or 0.0))
    q.coba = 1 if p.get("coba") else 0
    return q


class DeviceGraph:
    """A compiled connectome on the device (fb_graph). Shared read-only by any number of brains."""

    def __init__(self, g: Graph | None = None, *, N=None, indptr=None, indices=None, weights=None,
                 sign=None, _handle=None, _keep=None):
        self.L = nat.load()
        if _handle is not None:
            self.h, self.N, self.E, self._keep = _handle, N, int(_keep), None
            return
        if g is not None:
            N, indptr, indices, weights, sign = g.N, g.indptr, g.indices, g.weights, g.sign
        self.N = int(N)
        ip = np.ascontiguousarray(indptr, dtype=np.uint32)
        ix = np.ascontiguousarray(indices, dtype=np.uint32)
        w = np.ascontiguousarray(weights, dtype=np.float32)
        s = np.ascontiguousarray(sign, dtype=np.float32)
        self.E = int(ix.shape[0])
        h = C.c_void_p()
        nat.check(self.L.fb_graph_create(self.N, self.E, nat.ptr(ip), nat.ptr(ix), nat.ptr(w),
                                         nat.ptr(s), C.byref(h)))
        self.h = h
        self.indptr = ip  # LIFWasm exposes the CSR to callers (scripts/profile_fly.mjs:19)

    def shared(self, weights, sign) -> "DeviceGraph":
        """Same topology, its own weights and sign (per-trial gains baked in, as outScale)."""
        w = np.ascontiguousarray(weights, dtype=np.float32)
        s = np.ascontiguousarray(sign, dtype=np.float32)
        h = C.c_void_p()
        nat.check(self.L.fb_graph_create_shared(self.h, nat.ptr(w), nat.ptr(s), C.byref(h)))
        g = DeviceGraph(N=self.N, _handle=h, _keep=self.E)
        g.indptr = getattr(self, "indptr", None)
        return g

    def compile(self, counts, pre_sign, p: dict, in_scale=None, out_scale=None, sensory_mask=None,
                edge_gain=None) -> "DeviceGraph":
        """writeGraph (src/lifwasm.js:14-34) on the device over this graph's topology.

        counts, edge_gain: per edge; pre_sign, in_scale, out_scale (type gain), sensory_mask: per
        neuron. Arrays may be numpy (host) or torch CUDA tensors. p supplies wSyn, inhGain,
        minSyn and preInh (merged over DEFAULTS)."""
        q = dict(DEFAULTS, **p)
        cp = nat.FbCompileParams(float(q["wSyn"]), float(q["inhGain"]), float(q["minSyn"]), float(q["preInh"] or 0))
        keep = []

        def arr(x, dt):
            if x is None:
                return None
            if hasattr(x, "data_ptr"):
                keep.append(x)
                return x
            y = np.ascontiguousarray(x, dtype=dt)
            keep.append(y)
            return y

        h = C.c_void_p()
        nat.check(self.L.fb_graph_compile(
            self.h, nat.ptr(arr(counts, np.float32)), nat.ptr(arr(pre_sign, np.float32)),
            nat.ptr(arr(in_scale, np.float32)), nat.ptr(arr(out_scale, np.float32)),
            nat.ptr(arr(sensory_mask, np.uint8)), nat.ptr(arr(edge_gain, np.float32)), C.byref(cp), C.byref(h)))
        g = DeviceGraph(N=self.N, _handle=h, _keep=self.E)
        g.indptr = getattr(self, "indptr", None)
        return g

    def read(self):
        """(weights f32[E], sign f32[N]) as the device holds them."""
        w = np.zeros(self.E, dtype=np.float32)
        s = np.zeros(self.N, dtype=np.float32)
        nat.check(self.L.fb_graph_read(self.h, nat.ptr(w), nat.ptr(s)))
        return w, s

    def set_sign(self, sign):
        s = np.ascontiguousarray(sign, dtype=np.float32)
        nat.check(self.L.fb_graph_set_sign(self.h, nat.ptr(s)))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.fb_graph_destroy(h)
            self.h = None


class BrainBatch:
    """B brains (independent trials) on the device, stepped together by one persistent launch."""

    def __init__(self, graphs, params, seeds, mode: int = nat.FB_DELIVER_EXACT):
        self.L = nat.load()
        graphs = list(graphs)
        self.B = len(graphs)
        self.graphs = graphs
        if isinstance(params, dict):
            params = [params] * self.B
        self.p = [dict(DEFAULTS, **q) for q in params]
        arr = (nat.FbParams * self.B)(*[make_params(q) for q in self.p])
        gh = (C.c_void_p * self.B)(*[g.h.value if isinstance(g.h, C.c_void_p) else g.h for g in graphs])
        sd = np.ascontiguousarray(seeds, dtype=np.uint32)
        h = C.c_void_p()
        nat.check(self.L.fb_brains_create(gh, self.B, arr, C.sizeof(nat.FbParams), nat.ptr(sd), C.byref(h)))
        self.h = h
        self.N = [g.N for g in graphs]
        if mode != nat.FB_DELIVER_EXACT:
            self.set_mode(mode)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.fb_brains_destroy(h)
            self.h = None

    def set_mode(self, mode: int):
        nat.check(self.L.fb_brains_set_mode(self.h, int(mode)))

    def set_schedule(self, schedule: int):
        """FB_SCHEDULE_AUTO / _GRID / _LAGGED (fb_brains_set_schedule)."""
        nat.check(self.L.fb_brains_set_schedule(self.h, int(schedule)))

    def last_schedule(self) -> int:
        x = C.c_int32()
        nat.check(self.L.fb_last_schedule(self.h, C.byref(x)))
        return x.value

    def set_tuning(self, blocks_per_sm: int = 0, item_chunks: int = 0, sub_grab: int = 0,
                   timeout_us: int = 0, lag_driven_blocks: int | None = None):
        """Launch shape of the grid schedule, the bound of device-side waits and the delay-scheduled
        kernel's driven blocks (fb_brains_set_tuning); 0 keeps a knob (lag_driven_blocks: None
        keeps it, 0 makes it automatic)."""
        ldb = self.tuning()["lag_driven_blocks"] if lag_driven_blocks is None else int(lag_driven_blocks)
        t = nat.FbTuning(int(blocks_per_sm), int(item_chunks), 0, 0, int(sub_grab), int(timeout_us), ldb, 0)
        nat.check(self.L.fb_brains_set_tuning(self.h, C.byref(t)))

    def tuning(self) -> dict:
        t = nat.FbTuning()
        nat.check(self.L.fb_brains_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in nat.FbTuning._fields_}

    def trip_wait(self, step: int):
        """Test hook (fb_debug_trip_wait): the next delay-scheduled launch waits, at `step`, on a
        flag nothing sets, and ends with FB_ETIMEOUT after the timeout; -1 disarms."""
        nat.check(self.L.fb_debug_trip_wait(self.h, int(step)))

    def step(self, nsteps: int = 1) -> np.ndarray:
        out = np.zeros(self.B, dtype=np.int32)
        nat.check(self.L.fb_step(self.h, int(nsteps), nat.ptr(out)))
        return out

    def step_uneven(self, steps) -> np.ndarray:
        st = np.ascontiguousarray(steps, dtype=np.int32)
        out = np.zeros(self.B, dtype=np.int32)
        nat.check(self.L.fb_step_uneven(self.h, nat.ptr(st), nat.ptr(out)))
        return out

    def last_ms(self) -> float:
        ms = C.c_float()
        nat.check(self.L.fb_last_step_ms(self.h, C.byref(ms)))
        return ms.value

    def profile(self, on: bool = True):
        nat.check(self.L.fb_profile(self.h, 1 if on else 0))

    def phase_times(self) -> dict:
        """Accumulated per-phase milliseconds since profile(True): the grid kernel's phases (grid
        block 0's view) or, for the delay-scheduled kernel, the slots fb_phase_times documents."""
        ms = (C.c_double * 12)()
        nat.check(self.L.fb_phase_times(self.h, ms, 12))
        return dict(zip(("serial", "deliver", "barrier1", "update", "barrier2", "ctl_head",
                         "ctl_loads", "ctl_draw", "ctl_emit", "ctl_tail", "lag_publisher", "lag_helper"), list(ms)))

    def record(self, cap_steps: int, cap_spikes: int = 0):
        nat.check(self.L.fb_record(self.h, int(cap_steps), int(cap_spikes)))

    def spike_log(self, b: int, cap_steps: int, cap_spikes: int = 0):
        """(per-step fired counts, concatenated fired lists) recorded for brain b."""
        ns, nk = C.c_int64(), C.c_int64()
        nat.check(self.L.fb_spike_log(self.h, b, None, 0, None, 0, C.byref(ns), C.byref(nk)))
        counts = np.zeros(min(ns.value, cap_steps), dtype=np.int32)
        raster = np.zeros(min(nk.value, cap_spikes), dtype=np.int32)
        nat.check(self.L.fb_spike_log(self.h, b, nat.ptr(counts), counts.shape[0], nat.ptr(raster),
                                      raster.shape[0], C.byref(ns), C.byref(nk)))
        return counts, raster

    def fired(self, b: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        """The last step's fired list. out: an int32 buffer of capacity N (e.g. pinned host
        memory) read in one call; the result is a view of its first entries."""
        n = C.c_int32()
        if out is not None:
            if out.dtype != np.int32 or not out.flags.c_contiguous or out.shape[0] < self.N[b]:
                raise ValueError("fired: out must be a contiguous int32 array of at least N entries")
            nat.check(self.L.fb_fired(self.h, b, nat.ptr(out), out.shape[0], C.byref(n)))
            return out[:n.value]
        nat.check(self.L.fb_fired(self.h, b, None, 0, C.byref(n)))
        res = np.zeros(n.value, dtype=np.int32)
        nat.check(self.L.fb_fired(self.h, b, nat.ptr(res), n.value, C.byref(n)))
        return res

    def ring(self, b: int = 0):
        """Brain b's delay ring: (lists [nslots, N], counts [nslots], head); slot head is
        delivered next, and the slots after it hold the spikes still in flight."""
        q = self.p[b]
        ns = max(1, int(math.floor(q["delay"] / q["dt"] + 0.5))) + 1  # src/lifwasm.js:39
        lists = np.zeros(ns * self.N[b], dtype=np.int32)
        counts = np.zeros(ns, dtype=np.int32)
        head = C.c_int32()
        nat.check(self.L.fb_ring_read(self.h, b, nat.ptr(lists), nat.ptr(counts), C.byref(head)))
        return lists.reshape(ns, self.N[b]), counts, int(head.value)

    def _list(self, fn, b, idx, vals):
        idx = np.ascontiguousarray(np.atleast_1d(idx), dtype=np.int32)
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(vals, dtype=np.float64), idx.shape))
        nat.check(fn(self.h, b, nat.ptr(idx), nat.ptr(v), idx.shape[0]))

    def set_drive(self, b, idx, hz):
        self._list(self.L.fb_set_drive, b, idx, hz)

    def set_bias(self, b, idx, mv):
        self._list(self.L.fb_set_bias, b, idx, mv)

    def set_thr(self, b, idx, mv):
        self._list(self.L.fb_set_thr, b, idx, mv)

    def add_g(self, b, idx, e, i=None):
        idx = np.ascontiguousarray(np.atleast_1d(idx), dtype=np.int32)
        ev = np.ascontiguousarray(np.broadcast_to(np.asarray(e, dtype=np.float64), idx.shape))
        iv = None if i is None else np.ascontiguousarray(np.broadcast_to(np.asarray(i, dtype=np.float64), idx.shape))
        nat.check(self.L.fb_add_g(self.h, b, nat.ptr(idx), nat.ptr(ev), nat.ptr(iv), idx.shape[0]))

    def pulse(self, b, idx, mv):
        self._list(self.L.fb_pulse, b, idx, mv)

    def reset(self, b: int = -1):
        nat.check(self.L.fb_reset(self.h, int(b)))

    def set_background(self, b, rate_hz, amp_mv):
        nat.check(self.L.fb_set_background(self.h, b, float(rate_hz), float(amp_mv)))

    def set_params(self, b, params: dict):
        """New header constants for brain b from the next step on (fb_set_params)."""
        merged = dict(DEFAULTS, **params)
        q = make_params(merged)
        nat.check(self.L.fb_set_params(self.h, b, C.byref(q)))
        self.p[b] = merged

    def read(self, field: str, b: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        """A state field of brain b; out: a contiguous destination of N entries (e.g. pinned)."""
        dt = np.uint32 if field == "spikeCount" else np.float32
        if out is None:
            out = np.zeros(self.N[b], dtype=dt)
        elif out.dtype != dt or not out.flags.c_contiguous or out.shape[0] != self.N[b]:
            raise ValueError(f"read: out must be a contiguous {np.dtype(dt).name} array of N entries")
        nat.check(self.L.fb_read(self.h, nat.FIELDS[field], b, nat.ptr(out)))
        return out

    def write(self, field: str, b: int, values):
        dt = np.uint32 if field == "spikeCount" else np.float32
        v = np.ascontiguousarray(values, dtype=dt)
        nat.check(self.L.fb_write(self.h, nat.FIELDS[field], b, nat.ptr(v)))

    def scalars(self, b: int = 0) -> dict:
        head, nf, ls, nd = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        rng, sd = C.c_uint32(), C.c_int64()
        nat.check(self.L.fb_scalars(self.h, b, C.byref(head), C.byref(rng), C.byref(nf), C.byref(ls),
                                    C.byref(nd), C.byref(sd)))
        return dict(head=head.value, rng=rng.value, nFired=nf.value, lastSlot=ls.value,
                    nDriven=nd.value, stepsDone=sd.value)


class LIFCuda:
    """Drop-in for LIFWasm (src/lifwasm.js:36-87) on the GB300 step kernel: one brain."""

    def __init__(self, graph, params=None, seed: int = 1, N=None):
        if isinstance(graph, Graph):
            graph = DeviceGraph(graph)
        self.graph = graph
        self.N = graph.N
        self.p = dict(DEFAULTS, **(params or {}))
        self.nslots = max(1, int(math.floor(self.p["delay"] / self.p["dt"] + 0.5))) + 1
        self._batch = BrainBatch([graph], self.p, [seed])
        self.drivenSet: dict[int, None] = {}
        self.t = 0.0

    # setters (src/lifwasm.js:69-77)
    def setBackground(self, rate_hz, amp_mv):
        self.p["bgRate"], self.p["bgAmp"] = rate_hz, amp_mv
        self._batch.set_background(0, rate_hz, amp_mv)

    def setDriveOne(self, i, rate):
        self._batch.set_drive(0, [int(i)], [rate])
        if rate > 0:
            self.drivenSet.setdefault(int(i), None)
        else:
            self.drivenSet.pop(int(i), None)

    def setDrive(self, ix, rate):
        ix = np.atleast_1d(np.asarray(ix, dtype=np.int32))
        self._batch.set_drive(0, ix, rate)
        for i in ix.tolist():
            if rate > 0:
                self.drivenSet.setdefault(i, None)
            else:
                self.drivenSet.pop(i, None)

    def setBias(self, ix, mv):
        self._batch.set_bias(0, ix, mv)

    def setThr(self, i, mv):
        self._batch.set_thr(0, [int(i)], [mv])

    def setThrList(self, ix, mv):
        """setThr over a list in one host write (mv: one value or one per index), as a loop of
        setThr calls in list order would leave it."""
        self._batch.set_thr(0, np.asarray(ix, np.int32), mv)

    # LIFGpu extras (src/lifgpu.js:348-362)
    def setParams(self, q: dict):
        """Merged into the parameters; the header constants follow from the next step (the ring
        depth round(delay/dt)+1 must stay)."""
        merged = dict(self.p, **q)
        self._batch.set_params(0, merged)
        self.p = merged

    def flush(self):
        """Nothing to submit: queued writes apply before the next step."""

    def destroy(self):
        self._batch = None

    def addG(self, i, e, ii=0.0):
        self._batch.add_g(0, [int(i)], [e], [ii or 0.0])

    def pulse(self, ix, mv):
        self._batch.pulse(0, ix, mv)

    def wake(self, *a):
        pass

    def reset(self):
        self._batch.reset(0)
        self.t = 0.0

    def step(self) -> np.ndarray:
        """One step; the fired list in ring order (what LIFWasm.step's view holds)."""
        self._batch.step(1)
        self.t += self.p["dt"]
        return self._batch.fired(0)

    def run(self, nsteps: int) -> int:
        """nsteps steps in one launch; returns the last step's fired count."""
        nf = self._batch.step(nsteps)
        self.t += nsteps * self.p["dt"]
        return int(nf[0])

    @property
    def nAwake(self):
        return self.N

    def __getattr__(self, name):
        if name in nat.FIELDS:
            return self._batch.read(name, 0)
        raise AttributeError(name)
