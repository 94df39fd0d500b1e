"""The calibrated whole-CNS brain (src/brainmodel.js:7-100, src/brainsetup.js:10-18 and :70-78)
built from the connectome tables (flybrain.connectome), compiled and stepped on the GPU.

  region_size_ref      each neuron's reference volume: the median of its region (optic lobe,
                       central brain, nerve cord) (src/ratenet.js:22-31)
  brain_scales         inScale = min(boostCap, s^-sizeAlpha) (x vncGain in the nerve cord) with
                       s = clamp(size / regional median, 1/maxSizeScale, maxSizeScale), and the
                       sensory mask (superclass name containing "sensory") (src/brainmodel.js:8-19)
  class_physiology     Kenyon cells: threshold offset kcThreshold; lamina L1-L5: tonic bias
                       laminaBias (src/brainmodel.js:22-31)
  modulatory_sign      with neuromodulation on, octopaminergic neurons send no fast synapses
                       (src/brainmodel.js:34-43)
  type_gains           the outgoing weight scale (outScale): per-type and per-class multipliers, a
                       seeded lognormal individual, a fitted per-neuron log-gain table
                       (src/brainmodel.js:63-100)
  brain_graph          allocBrainMemory's writeGraph, on the device (src/brainsetup.js:10-18)
  attach_brain         one brain on that graph with the class physiology applied
                       (src/brainsetup.js:70-78)
  create_brain         createBrain (src/brainmodel.js:44-46): both steps for one brain

Values are computed as the reference computes them: float64 arithmetic, stored to float32 where the
reference stores to a Float32Array (inScale once; outScale after every multiply). Math.pow, exp,
log and cos come from the host's C library here and from the JavaScript engine there; both are
within an ulp in float64, so a stored float32 can differ from the reference's in rare ties.
The neuromodulation controller that runs beside a calibrated brain (src/sim/neuromod.js, the
octopamine threshold field) is flybrain.neuromod.
"""
from __future__ import annotations

import math
import re

import numpy as np

from .connectome import pre_sign as table_sign

# src/brainmodel.js:7
BRAIN_DEFAULTS = dict(laminaBias=9.0, kcThreshold=0.0, wSyn=0.3, sizeAlpha=0.5, minSyn=5, adaptInc=0.0, depU=0.0,
                      maxSizeScale=20.0, boostCap=1.0)
_REGION0 = re.compile(r"^(ol_|visual_projection|visual_centrifugal)")
_REGION2 = re.compile(r"^(vnc_|descending|ascending|sensory_ascending|sensory_descending|efferent_)")
_LAMINA = re.compile(r"^L[1-5]$")
_REGEX_CHARS = re.compile(r"[\\^$*+?()\[\]{}|]")


def _js_str(x) -> str:
    """A table entry as a JavaScript regular expression test sees it (a missing entry is 'undefined')."""
    return "undefined" if x is None else str(x)


def region_of(name: str) -> int:
    """0 optic lobe, 1 central brain, 2 nerve cord, from the superclass name (src/ratenet.js:22)."""
    name = _js_str(name)
    return 0 if _REGION0.match(name) else 2 if _REGION2.match(name) else 1


def region_size_ref(superclass_names, sc, size):
    """(ref f32[N], medians [3], region u8[N]): per region, the element at index len//2 of the
    sorted positive sizes, 1 for a region with none (src/ratenet.js:23-31)."""
    sc = np.asarray(sc, np.int64)
    size = np.asarray(size, np.float32)
    reg_of_sc = np.array([region_of(n) for n in superclass_names] or [1], np.uint8)
    region = np.where(sc < len(superclass_names), reg_of_sc[np.minimum(sc, reg_of_sc.shape[0] - 1)], 1).astype(np.uint8)
    med = []
    for r in range(3):
        b = np.sort(size[(region == r) & (size > 0)])
        m = float(b[b.shape[0] >> 1]) if b.shape[0] else 0.0
        med.append(m or 1.0)
    return np.asarray(med, np.float32)[region], med, region


def brain_scales(c: dict, size, opts: dict | None = None):
    """(inScale f32[N], sensoryMask u8[N], region u8[N]) (src/brainmodel.js:8-19)."""
    o = dict(BRAIN_DEFAULTS, **(opts or {}))
    names = list(c["meta"].get("superclasses", []))
    ref, _, region = region_size_ref(names, c["sc"], size)
    size = np.asarray(size, np.float32).astype(np.float64)
    mx = float(o["maxSizeScale"])
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(size > 0, np.minimum(mx, np.maximum(1.0 / mx, size / ref.astype(np.float64))), 1.0)
        in_scale = np.minimum(float(o["boostCap"]), np.power(s, -float(o["sizeAlpha"])))
    if o.get("vncGain"):
        in_scale = in_scale * np.where(region == 2, float(o["vncGain"]), 1.0)
    sc = np.asarray(c["sc"], np.int64)
    sens = np.array([1 if "sensory" in _js_str(n) else 0 for n in names] + [0], np.uint8)
    mask = sens[np.where(sc < len(names), sc, len(names))]
    return in_scale.astype(np.float32), mask, region


def class_physiology(c: dict, opts: dict | None = None):
    """((Kenyon cell indices, threshold offset), (lamina L1-L5 indices, bias)) as
    applyClassPhysiology sets them (src/brainmodel.js:22-31)."""
    o = dict(BRAIN_DEFAULTS, **(opts or {}))
    classes = list(c["meta"].get("classes", []))
    types = list(c["meta"].get("types", []))
    cls = np.asarray(c["cls"], np.int64)
    kc = np.array([i for i in range(c["N"]) if cls[i] < len(classes) and classes[cls[i]] == "Kenyon_Cell"], np.int32)
    lam = np.array([i for i in range(c["N"]) if _LAMINA.match(_js_str(types[i] if i < len(types) else None))], np.int32)
    return (kc, float(o["kcThreshold"])), (lam, float(o["laminaBias"]))


def modulatory_sign(c: dict, pre_sign, opts: dict | None = None):
    """The per-neuron sign with octopaminergic neurons (type 'OA-...') silenced when neuromodulation
    is on, unless oaMode is 'synFast'; None (the transmitter table) when nothing changes and no
    sign was given (src/brainmodel.js:34-43)."""
    o = dict(BRAIN_DEFAULTS, **(opts or {}))
    if not o.get("neuromod"):
        return pre_sign
    s = np.array(table_sign(c) if pre_sign is None else pre_sign, np.float32)
    if o.get("oaMode") == "synFast":
        return s
    types = list(c["meta"].get("types", []))
    for i in range(min(c["N"], len(types))):
        if _js_str(types[i]).startswith("OA-"):
            s[i] = 0.0
    return s


def _mulberry32_lognormal(N: int, sigma: float, seed: int) -> np.ndarray:
    """exp(sigma * z) for N draws of the reference's seeded generator and Box-Muller transform
    (src/brainmodel.js:85-90), in float64."""
    M = 0xFFFFFFFF
    # (seed * 2654435761) | 0: the product in double (rounded above 2^53), then modulo 2^32
    a = int(math.fmod(math.floor(float(seed) * 2654435761.0), 4294967296.0)) & M

    def rnd():
        nonlocal a
        a = (a + 0x6D2B79F5) & M
        t = ((a ^ (a >> 15)) * (1 | a)) & M
        t = ((t + (((t ^ (t >> 7)) * (61 | t)) & M)) & M) ^ t
        return ((t ^ (t >> 14)) & M) / 4294967296.0

    out = np.empty(N, np.float64)
    for i in range(N):
        u = rnd()
        v = rnd()
        if u <= 0:
            u = 1e-9
        out[i] = math.exp(sigma * math.sqrt(-2 * math.log(u)) * math.cos(2 * math.pi * v))
    return out


def type_gains(c: dict, opts: dict | None = None):
    """outScale f32[N], or None when no gain is set (src/brainmodel.js:63-100).

    opts: typeGain {type name or regular-expression source: gain}, neuronGain {sigma, seed},
    classGain {class name: gain}, neuronGainTable (log gains, per neuron or {index: log gain}).
    Each multiply is float64 stored to float32, in the reference's order."""
    o = opts or {}
    spec, cspec, table = o.get("typeGain"), o.get("classGain"), o.get("neuronGainTable")
    keys = [k for k in (spec or {}) if spec[k] != 1]
    ckeys = [k for k in (cspec or {}) if cspec[k] != 1]
    ng = o.get("neuronGain") or {}
    if not keys and not ckeys and not ng.get("sigma") and table is None:
        return None
    N = int(c["N"])
    types = list(c["meta"].get("types", []))
    tname = [_js_str(types[i] if i < len(types) else None) for i in range(N)]
    g = np.ones(N, np.float32)

    def mul(mask, f):
        g[mask] = (g[mask].astype(np.float64) * np.asarray(f, np.float64)[mask if np.ndim(f) else ()]).astype(np.float32)

    for k in keys:
        pat = re.compile(f"^(?:{k})$") if _REGEX_CHARS.search(k) else None
        m = np.array([bool(pat.match(t)) if pat else (i < len(types) and types[i] == k) for i, t in enumerate(tname)],
                     bool)
        mul(m, float(spec[k]))
    if ng.get("sigma"):
        mul(np.ones(N, bool), _mulberry32_lognormal(N, float(ng["sigma"]), int(ng.get("seed", 1))))
    if ckeys:
        classes = list(c["meta"].get("classes", []))
        cls = np.asarray(c["cls"], np.int64)
        f = np.ones(N, np.float64)
        m = np.zeros(N, bool)
        for i in range(N):
            name = classes[cls[i]] if cls[i] < len(classes) else None
            if name in cspec:
                f[i], m[i] = float(cspec[name]), True
        mul(m, f)
    if table is not None:
        if isinstance(table, dict):
            for k, v in table.items():
                i = int(k)
                g[i] = np.float32(float(g[i]) * math.exp(float(v)))
        else:
            t = np.zeros(N, np.float64)
            tv = np.asarray(table, np.float64)[:N]
            t[:tv.shape[0]] = tv
            m = (t != 0) & ~np.isnan(t)
            f = np.ones(N, np.float64)
            f[m] = np.exp(t[m])
            mul(m, f)
    return g


def brain_graph(c: dict, size, sign=None, opts: dict | None = None, eye_pairs=None):
    """allocBrainMemory's graph (src/brainsetup.js:10-18) compiled on the device: returns
    (DeviceGraph, LIF parameters, scales dict). eye_pairs lists the optic-lobe neurons that the
    visual system drives; they join the sensory mask."""
    from .brain import DEFAULTS, DeviceGraph
    o = dict(BRAIN_DEFAULTS, **(opts or {}))
    in_scale, mask, region = brain_scales(c, size, o)
    if eye_pairs is not None:
        mask[np.asarray(eye_pairs, np.int64)] = 1
    s = modulatory_sign(c, sign, o)
    out_scale = type_gains(c, o)
    p = dict(DEFAULTS, **{k: v for k, v in o.items() if k in DEFAULTS})
    topo = DeviceGraph(N=c["N"], indptr=c["indptr"], indices=c["indices"], weights=np.zeros(c["E"], np.float32),
                       sign=np.zeros(c["N"], np.float32))
    edge_gain = o.get("edgeGain")
    dg = topo.compile(np.asarray(c["counts"], np.float32), table_sign(c) if s is None else s, p, in_scale=in_scale,
                      out_scale=out_scale, sensory_mask=mask, edge_gain=edge_gain)
    return dg, p, dict(in_scale=in_scale, sensory_mask=mask, region=region, pre_sign=s, out_scale=out_scale)


def attach_brain(dg, p: dict, c: dict, opts: dict | None = None, seed: int = 1):
    """A LIFCuda brain on the compiled graph with the class physiology applied (src/brainsetup.js:77-78)."""
    from .brain import LIFCuda
    brain = LIFCuda(dg, p, seed=seed)
    (kc, kv), (lam, lv) = class_physiology(c, opts)
    if kc.shape[0]:
        brain.setThrList(kc, kv)
    if lam.shape[0]:
        brain.setBias(lam, lv)
    return brain


def create_brain(c: dict, size, opts: dict | None = None, pre_sign=None, seed: int = 1):
    """createBrain (src/brainmodel.js:44-46): the calibrated graph and one brain on it; gradedSign
    False drops a given graded sign for the transmitter table."""
    o = dict(BRAIN_DEFAULTS, **(opts or {}))
    dg, p, scales = brain_graph(c, size, None if o.get("gradedSign") is False else pre_sign, o)
    return attach_brain(dg, p, c, o, seed), scales
