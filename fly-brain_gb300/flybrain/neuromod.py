"""Neuromodulation over a brain (src/sim/neuromod.js): haemolymph sugar sets AKH and, through the
glucose-sensing IPCs, insulin; both drive the octopaminergic (OA) neurons, whose low-pass firing
rate is the octopamine they release. Released octopamine acts through G-protein receptors, not
fast synapses: under the shipped operator (oaMode 'thrField') it lowers the spike threshold of
the neurons the OA cells synapse onto, saturating in synapses x Hz; 'thrTyped' restricts that to a
versioned type list, 'gainField' scales the outgoing gain (the graph's per-neuron sign) of typed
sets instead, 'synFast' leaves OA its fast synapses and no field. OA neurons and IPCs also get a
slow afterhyperpolarisation (threshold rising with their own rate).

The controller is host logic between brain steps, as in the reference: every millisecond it adds
conductances (addG), every 10 ms it reads the modulatory cells' spike counts and resets their
thresholds, every 50 ms it recomputes the field and writes the targets' thresholds (setThr) or the
graph's signs. It drives any object with the LIFWasm surface (LIFCuda on the GPU, the oracle
brain on the host) and keeps the reference's number formats: the per-cell and per-target arrays
are float32 (each update formed in double and stored once), the AKH and insulin levels double.
"""
from __future__ import annotations

import math
import re

import numpy as np

# src/sim/neuromod.js:27-50
NEUROMOD = dict(akhHalf=0.4, akhWidth=0.15, akhTau=5000.0, ipcHalf=0.4, ipcWidth=0.15, ipcDrive=4.0, ipcFed=5.0,
                dilpTau=10000.0, akhDrive=3.0, insDrive=1.0, oaTau=2000.0, sfa=0.5, oaFed=2.0, oaStarved=12.0,
                targetShift=2.0, targetHalf=400.0, locoDrive=6.0, oaMode="thrField", gainMax=2.0, oaTargets=None)
AKHR_TYPES = re.compile(r"^OA-(VUMa|VPM)")
OPTIC_OA_TYPES = re.compile(r"^OA-(AL2i|ASM)")
_REGEX_CHARS = re.compile(r"[\\^$*+?()\[\]{}|]")


def is_octopaminergic(t) -> bool:
    return t is not None and str(t).startswith("OA-")


def _sig(x, half, w):
    return 1.0 / (1.0 + math.exp(-(x - half) / w))


def _f32(x):
    return np.float32(x)


def _type_matcher(types, keys):
    pats = [re.compile(f"^(?:{k})$") if _REGEX_CHARS.search(k) else None for k in keys]

    def match(i):
        t = types[i] if i < len(types) else None
        s = "undefined" if t is None else str(t)
        return any(p.match(s) if p else t == k for p, k in zip(pats, keys))
    return match


class _SignIO:
    """The brain's writable per-neuron graph sign (s * wSyn): the compiled device graph's, or the
    host array of a brain that holds one."""

    def __init__(self, brain):
        g = getattr(brain, "graph", None)
        if g is not None and hasattr(g, "set_sign"):
            self.get = lambda: g.read()[1]
            self.set = g.set_sign
        elif getattr(brain, "sign", None) is not None:
            arr = brain.sign

            def put(v):
                arr[:] = v
            self.get = lambda: np.array(arr, np.float32)
            self.set = put
        else:
            raise ValueError("oaMode 'gainField' needs a writable per-neuron sign array")


class Neuromod:
    """src/sim/neuromod.js:53-170 over `brain`. data: the connectome tables (N, indptr, indices,
    counts or weights = synapse counts, meta.types; sc and meta.superclasses for gainField);
    calib: parsed neuromod.json ({oaThr, ipcThr}: resting thresholds by neuron index); block:
    'OA' | 'AKHR' | 'InR' | None."""

    def __init__(self, data, brain, calib=None, block=None, min_syn=5, params=None):
        self.P = dict(NEUROMOD, **(params or {}))
        self.block, self.brain = block, brain
        types = list(data["meta"].get("types", []))
        N = int(data["N"])
        t_of = lambda i: types[i] if i < len(types) else None  # noqa: E731
        oa = [i for i in range(N) if is_octopaminergic(t_of(i))]
        ipc = [i for i in range(N) if t_of(i) == "IPC"]
        self.cells = np.array(oa + ipc, np.int32)
        self.nOA = len(oa)
        self.akhr_pos = np.array([n for n, i in enumerate(oa) if AKHR_TYPES.match(str(t_of(i)))], np.int32)
        self.optic = np.array([i for i in oa if OPTIC_OA_TYPES.match(str(t_of(i)))], np.int32)
        self.akhr = np.array([oa[n] for n in self.akhr_pos], np.int32)
        self.ipc = np.array(ipc, np.int32)
        cal = {}
        if calib:
            cal.update({int(k): v for k, v in (calib.get("oaThr") or {}).items()})
            cal.update({int(k): v for k, v in (calib.get("ipcThr") or {}).items()})
        thr = np.asarray(brain.thr, np.float32)
        self.base = np.array([cal.get(int(i), thr[i]) for i in self.cells], np.float32)
        self.r = np.array([self.P["oaFed"] if n < self.nOA else self.P["ipcFed"] for n in range(len(self.cells))],
                          np.float32)
        self.c = self.r[:self.nOA]  # octopamine release per OA neuron (a view, as in the reference)
        sc = np.asarray(brain.spikeCount)
        self.last = sc[self.cells].astype(np.uint32)
        # octopamine targets: synapse counts from each OA neuron, the fast graph's minimum applied
        indptr, indices = np.asarray(data["indptr"]), np.asarray(data["indices"])
        w = np.asarray(data["counts"] if "counts" in data else data["weights"])
        t_ix: dict[int, int] = {}
        self.rows = []
        for j in oa:
            row = []
            for k in range(int(indptr[j]), int(indptr[j + 1])):
                if w[k] < min_syn:
                    continue
                q = int(indices[k])
                if q not in t_ix:
                    t_ix[q] = len(t_ix)
                row += [t_ix[q], int(w[k])]
            self.rows.append(np.array(row, np.int64))
        self.targets = np.array(list(t_ix.keys()), np.int32)
        self.x = np.zeros(len(self.targets), np.float32)
        self.shift = np.zeros(len(self.targets), np.float32)
        self.thr0 = thr[self.targets].copy() if len(self.targets) else np.zeros(0, np.float32)
        cell_set = set(self.cells.tolist())
        self.is_cell = np.array([1 if q in cell_set else 0 for q in self.targets.tolist()], np.uint8)
        self.cell_target = np.array([t_ix.get(int(i), -1) for i in self.cells], np.int32)
        self.akh, self.dilp, self.t = 0.0, 1.0, 0.0
        self.adapt = None  # calibration: {"eta": ...} moves the cells' resting thresholds to their fed rates
        self.oa_mode = self.P["oaMode"]
        T = self.P["oaTargets"]
        self.field_mask = None
        if self.oa_mode == "thrTyped":
            if not T or not T.get("thrTyped"):
                raise ValueError("oaMode 'thrTyped' requires params.oaTargets (oa_targets.json)")
            m = _type_matcher(types, T["thrTyped"])
            self.field_mask = np.array([1 if m(int(q)) else 0 for q in self.targets], np.uint8)
        self.sign_io = None
        if self.oa_mode == "gainField":
            if not T or not T.get("gainField"):
                raise ValueError("oaMode 'gainField' requires params.oaTargets (oa_targets.json)")
            sup = list(data["meta"].get("superclasses", []))
            in_sup = {sup.index(s) if s in sup else -1 for s in T["gainField"]["superclasses"]}
            m = _type_matcher(types, T["gainField"].get("types") or [])
            scs = np.asarray(data["sc"])
            self.field_mask = np.array([1 if int(scs[q]) in in_sup or m(int(q)) else 0 for q in self.targets], np.uint8)
            self.sign_io = _SignIO(brain)
            self.sign0 = np.array(self.sign_io.get(), np.float32)
            self.sign = self.sign0.copy()
        self.set_cell_thr()

    def reset(self):
        """After brain.reset() (spike counts cleared): back to the fed steady state."""
        self.last = np.asarray(self.brain.spikeCount)[self.cells].astype(np.uint32)
        self.r[:self.nOA] = self.P["oaFed"]
        self.r[self.nOA:] = self.P["ipcFed"]
        self.akh, self.dilp, self.t = 0.0, 1.0, 0.0
        if self.sign_io is not None:
            self.sign = self.sign0.copy()
            self.sign_io.set(self.sign)
        self.set_cell_thr()

    def update(self, dt_ms, sugar, loco=0.0):
        """One millisecond; sugar = haemolymph sugar (energy 0..1); loco = locomotor state 0..1."""
        P, B = self.P, self.brain
        self.t += dt_ms
        t = self.t
        self.akh += (_sig(-sugar, -P["akhHalf"], P["akhWidth"]) - self.akh) * dt_ms / P["akhTau"]
        g_ipc = P["ipcDrive"] * _sig(sugar, P["ipcHalf"], P["ipcWidth"]) * dt_ms
        for i in self.ipc:
            B.addG(int(i), g_ipc)
        akh = 0.0 if self.block == "AKHR" else self.akh
        ins = 0.0 if self.block == "InR" else self.dilp
        gA, gI = P["akhDrive"] * akh * dt_ms, P["insDrive"] * ins * dt_ms
        for i in self.akhr:
            B.addG(int(i), gA, -gI)
        if loco > 0:
            gL = P["locoDrive"] * loco * dt_ms
            for i in self.optic:
                B.addG(int(i), gL)
        if t % 10 == 0:
            self.release(10)
        if t % 50 == 0 and self.block != "OA":
            self.modulate()

    def release(self, ms):
        P, B = self.P, self.brain
        k = ms / P["oaTau"]
        sc = np.asarray(B.spikeCount)
        for n in range(len(self.cells)):
            s = int(sc[self.cells[n]])
            rn = float(self.r[n])
            self.r[n] = _f32(rn + ((s - int(self.last[n])) * 1000 / ms - rn) * k)
            self.last[n] = s
        ipc = 0.0
        for n in range(self.nOA, len(self.cells)):
            ipc += float(self.r[n])
        if len(self.ipc):
            self.dilp += (min(1.5, ipc / len(self.ipc) / P["ipcFed"]) - self.dilp) * ms / P["dilpTau"]
        else:  # no IPCs in the tables: 0 / 0, as the reference's arithmetic gives
            self.dilp = float("nan")
        if self.adapt:
            e = self.adapt["eta"] * ms / 1000
            for n in range(len(self.cells)):
                fed = P["oaFed"] if n < self.nOA else P["ipcFed"]
                self.base[n] = _f32(float(self.base[n]) + e * math.log((float(self.r[n]) + 0.5) / (fed + 0.5)))
        self.set_cell_thr()

    def set_cell_thr(self):
        if not len(self.cells):
            return
        v = np.empty(len(self.cells), np.float64)
        for n in range(len(self.cells)):
            m = int(self.cell_target[n])
            v[n] = float(self.base[n]) + self.P["sfa"] * float(self.r[n]) - (0.0 if m < 0 else float(self.shift[m]))
        self._set_thr(self.cells, v)

    def _set_thr(self, idx, vals):
        B = self.brain
        if hasattr(B, "setThrList"):  # one list write (the same as setThr per element, in order)
            B.setThrList(idx, np.asarray(vals, np.float64))
        else:
            for i, v in zip(idx.tolist(), vals.tolist()):
                B.setThr(int(i), v)

    def modulate(self):
        """Octopamine's postsynaptic action under oaMode; x is per-target exposure in synapses x Hz."""
        P = self.P
        x = self.x
        x[:] = 0
        for n, row in enumerate(self.rows):
            c = float(self.c[n])
            if c <= 0:
                continue
            for m in range(0, len(row), 2):
                q = int(row[m])
                x[q] = _f32(float(x[q]) + int(row[m + 1]) * c)
        if self.oa_mode == "synFast":
            self.shift[:] = 0
            return
        mask = self.field_mask
        if self.oa_mode == "gainField":
            for m in range(len(x)):
                q = int(self.targets[m])
                self.shift[m] = 0
                xm = float(x[m])
                self.sign[q] = _f32(float(self.sign0[q]) * (1 + P["gainMax"] * xm / (xm + P["targetHalf"]))) \
                    if mask[m] else self.sign0[q]
            self.sign_io.set(self.sign)
            return
        idx, vals = [], []
        for m in range(len(x)):
            xm = float(x[m])
            self.shift[m] = _f32(P["targetShift"] * xm / (xm + P["targetHalf"])) if (mask is None or mask[m]) else 0
            if not self.is_cell[m]:
                idx.append(int(self.targets[m]))
                vals.append(float(self.thr0[m]) - float(self.shift[m]))
        if idx:
            self._set_thr(np.array(idx, np.int32), np.array(vals, np.float64))

    @property
    def oa_tone(self):
        """Mean octopamine release of the AKH-sensitive OA neurons (Hz), summed in order."""
        tot = 0.0
        for n in self.akhr_pos.tolist():
            tot += float(self.c[n])
        return tot / len(self.akhr_pos) if len(self.akhr_pos) else float("nan")

    @property
    def arousal(self):
        oa = self.P["oaFed"] if self.block == "OA" else self.oa_tone
        return max(0.0, min(1.0, (oa - self.P["oaFed"]) / (self.P["oaStarved"] - self.P["oaFed"])))

    def readout(self):
        return dict(akh=self.akh, dilp=self.dilp, oa=self.oa_tone, arousal=self.arousal)

    def thresholds(self):
        """Resting thresholds of the modulatory cells, in neuromod.json's form."""
        o = dict(oaThr={}, ipcThr={})
        for n, i in enumerate(self.cells.tolist()):
            (o["oaThr"] if n < self.nOA else o["ipcThr"])[str(i)] = round(float(self.base[n]), 3)
        return o
