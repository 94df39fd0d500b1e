"""The reference's preprocessed connectome tables (a data directory like its public/data), read
into the arrays the device graph compile takes.

Layouts (scripts/prep_graph.py:46-56, read by scripts/lib_node.mjs:3-13 and src/data.js):
  meta.json              {N, minWeight, edges, nts, superclasses, classes, types, instances}
  graph_w{minWeight}.bin u32 {N, E}; u32 indptr[N+1]; u32 indices[E]; u16 counts[E] (synapses per
                         connection, capped at 65535), rows sorted by target
  neurons.bin            u32 {N, 0}; i64 bodyIds[N]; f32 soma[N][3]; u32 indeg[N]; u32 outdeg[N];
                         u16 cls[N]; u8 nt[N]; u8 sc[N]; u8 side[N]
  neuron_size.bin        f32[N] (relative volume; <= 0 when unknown)
  ntsign.bin             f32[N] (transmitter sign, graded when unknown)

  graph.flyg / neurons.flyn the same graph and table range coded (src/codec/graph.js,
                         src/codec/neurons.js): what the web app loads (src/data.js:21-34); decoded
                         by the native library (fb_flyg_decode, fb_flyn_decode) into the arrays above

load_connectome(dir) returns the tables; to_device_graph(c, params, ...) compiles them on the GPU
the way writeGraph does (src/lifwasm.js:14-34) with the transmitter signs of src/lif.js:5.
"""
from __future__ import annotations

import json
import os

import numpy as np

EXC_SIGN = np.array([0, 1, -1, -1, 1, 1, 1, -1], np.float32)  # src/lif.js:5, by transmitter id


def _read(path, dtype, count, offset):
    a = np.fromfile(path, dtype=dtype, count=count, offset=offset)
    if a.shape[0] != count:
        raise ValueError(f"{path}: expected {count} x {np.dtype(dtype).name} at byte {offset}, file too short")
    return a


def load_graph(path: str, N: int | None = None) -> dict:
    """graph_w*.bin: {N, E, indptr u32[N+1], indices u32[E], counts u16[E]}, validated."""
    hdr = _read(path, np.uint32, 2, 0)
    n, E = int(hdr[0]), int(hdr[1])
    if N is not None and n != N:
        raise ValueError(f"{path}: N={n}, the metadata says {N}")
    off = 8
    indptr = _read(path, np.uint32, n + 1, off)
    off += (n + 1) * 4
    indices = _read(path, np.uint32, E, off)
    off += E * 4
    counts = _read(path, np.uint16, E, off)
    if indptr[0] != 0 or int(indptr[-1]) != E or np.any(np.diff(indptr.astype(np.int64)) < 0):
        raise ValueError(f"{path}: indptr is not a CSR offset array for {E} edges")
    if E and int(indices.max()) >= n:
        raise ValueError(f"{path}: target index out of range")
    return dict(N=n, E=E, indptr=indptr, indices=indices, counts=counts)


def load_flyg(path: str) -> dict:
    """graph.flyg decoded: {N, E, min_weight, indptr u32[N+1], indices u32[E], counts u16[E]}, the
    arrays of graph_w{min_weight}.bin (src/codec/graph.js:70-108)."""
    import ctypes as C
    from . import _native as nat
    L = nat.load()
    raw = np.fromfile(path, dtype=np.uint8)
    h = nat.FbFlygHeader()
    nat.check(L.fb_flyg_sizes(nat.ptr(raw), raw.shape[0], C.byref(h)))
    indptr = np.zeros(h.N + 1, np.uint32)
    indices = np.zeros(h.E, np.uint32)
    counts = np.zeros(h.E, np.uint16)
    nat.check(L.fb_flyg_decode(nat.ptr(raw), raw.shape[0], nat.ptr(indptr), nat.ptr(indices), nat.ptr(counts)))
    return dict(N=int(h.N), E=int(h.E), min_weight=int(h.min_weight), indptr=indptr, indices=indices, counts=counts)


def load_flyn(path: str) -> dict:
    """neurons.flyn decoded: {N, bodyIds, soma, cls, nt, sc, side} as in neurons.bin, soma NaN where
    absent (src/codec/neurons.js:25-37). In- and out-degrees follow from the graph."""
    import ctypes as C
    from . import _native as nat
    L = nat.load()
    raw = np.fromfile(path, dtype=np.uint8)
    n = C.c_uint32()
    nat.check(L.fb_flyn_count(nat.ptr(raw), raw.shape[0], C.byref(n)))
    N = int(n.value)
    out = dict(N=N, bodyIds=np.zeros(N, np.int64), soma=np.zeros((N, 3), np.float32), cls=np.zeros(N, np.uint16),
               nt=np.zeros(N, np.uint8), sc=np.zeros(N, np.uint8), side=np.zeros(N, np.uint8))
    nat.check(L.fb_flyn_decode(nat.ptr(raw), raw.shape[0], *(nat.ptr(out[k]) for k in
                                                              ("bodyIds", "soma", "cls", "nt", "sc", "side"))))
    return out


def load_neurons(path: str, N: int) -> dict:
    """neurons.bin: per-neuron annotations in the layout of scripts/prep_graph.py:54."""
    hdr = _read(path, np.uint32, 2, 0)
    if int(hdr[0]) != N:
        raise ValueError(f"{path}: N={int(hdr[0])}, expected {N}")
    off = 8
    out = {}
    for name, dt, k in (("bodyIds", np.int64, 1), ("soma", np.float32, 3), ("indeg", np.uint32, 1),
                        ("outdeg", np.uint32, 1), ("cls", np.uint16, 1), ("nt", np.uint8, 1),
                        ("sc", np.uint8, 1), ("side", np.uint8, 1)):
        a = _read(path, dt, N * k, off)
        out[name] = a.reshape(N, 3) if k == 3 else a
        off += N * k * np.dtype(dt).itemsize
    return out


def load_connectome(data_dir: str, min_weight: int | None = None) -> dict:
    """The whole table set of a data directory: meta, graph, neurons, and the optional per-neuron
    size and sign arrays (None when absent)."""
    with open(os.path.join(data_dir, "meta.json")) as f:
        meta = json.load(f)
    N = int(meta["N"])
    mw = int(min_weight if min_weight is not None else meta["minWeight"])
    gpath, fpath = os.path.join(data_dir, f"graph_w{mw}.bin"), os.path.join(data_dir, "graph.flyg")
    if not os.path.exists(gpath) and os.path.exists(fpath):  # the app's compressed copy
        f = load_flyg(fpath)
        if f["N"] != N or f["min_weight"] != mw:
            raise ValueError(f"graph.flyg holds N={f['N']}, minWeight={f['min_weight']}; asked for N={N}, minWeight={mw}")
        g = {k: f[k] for k in ("N", "E", "indptr", "indices", "counts")}
    else:
        g = load_graph(gpath, N)
    if "edges" in meta and min_weight is None and int(meta["edges"]) != g["E"]:
        raise ValueError(f"graph_w{mw} has {g['E']} edges, the metadata says {meta['edges']}")
    c = dict(meta=meta, min_weight=mw, **g)
    npath, fpath = os.path.join(data_dir, "neurons.bin"), os.path.join(data_dir, "neurons.flyn")
    if not os.path.exists(npath) and os.path.exists(fpath):
        t = load_flyn(fpath)
        if t["N"] != N:
            raise ValueError(f"neurons.flyn holds N={t['N']}, the metadata says {N}")
        t.pop("N")
        t["outdeg"] = np.diff(g["indptr"].astype(np.int64)).astype(np.uint32)
        t["indeg"] = np.bincount(g["indices"], minlength=N).astype(np.uint32)
        c.update(t)
    else:
        c.update(load_neurons(npath, N))
    for name, fn in (("size", "neuron_size.bin"), ("ntsign", "ntsign.bin")):
        p = os.path.join(data_dir, fn)
        c[name] = _read(p, np.float32, N, 0) if os.path.exists(p) else None
    return c


def write_connectome(data_dir: str, N: int, indptr, indices, counts, nt, min_weight: int = 3, extra: dict | None = None):
    """Writes a table set in the same layouts (for tests and for graphs made elsewhere)."""
    os.makedirs(data_dir, exist_ok=True)
    indptr = np.ascontiguousarray(indptr, np.uint32)
    indices = np.ascontiguousarray(indices, np.uint32)
    counts = np.ascontiguousarray(np.minimum(counts, 65535), np.uint16)
    E = int(indices.shape[0])
    with open(os.path.join(data_dir, f"graph_w{min_weight}.bin"), "wb") as f:
        for a in (np.array([N, E], np.uint32), indptr, indices, counts):
            f.write(a.tobytes())
    outdeg = np.diff(indptr.astype(np.int64)).astype(np.uint32)
    indeg = np.bincount(indices, minlength=N).astype(np.uint32)
    with open(os.path.join(data_dir, "neurons.bin"), "wb") as f:
        for a in (np.array([N, 0], np.uint32), np.arange(N, dtype=np.int64), np.zeros((N, 3), np.float32), indeg,
                  outdeg, np.zeros(N, np.uint16), np.ascontiguousarray(nt, np.uint8), np.zeros(N, np.uint8),
                  np.zeros(N, np.uint8)):
            f.write(np.ascontiguousarray(a).tobytes())
    meta = dict(N=int(N), minWeight=int(min_weight), edges=E, nts=["unknown", "acetylcholine", "gaba", "glutamate",
                                                                     "dopamine", "serotonin", "octopamine", "histamine"],
                superclasses=[], classes=[""], types=[""] * int(N))
    meta.update(extra or {})
    with open(os.path.join(data_dir, "meta.json"), "w") as f:
        json.dump(meta, f)


def pre_sign(c: dict, graded: bool = False) -> np.ndarray:
    """Per-neuron sign before wSyn: the transmitter table of src/lif.js:5, or the graded ntsign
    array when asked for and present."""
    if graded and c.get("ntsign") is not None:
        return np.asarray(c["ntsign"], np.float32)
    return EXC_SIGN[np.asarray(c["nt"], np.int64)]


def to_device_graph(c: dict, params: dict, in_scale=None, out_scale=None, sensory_mask=None, graded: bool = False):
    """Compiles the tables on the GPU as writeGraph does (src/lifwasm.js:14-34): a DeviceGraph
    ready for BrainBatch / LIFCuda."""
    from .brain import DeviceGraph
    topo = DeviceGraph(N=c["N"], indptr=c["indptr"], indices=c["indices"], weights=np.zeros(c["E"], np.float32),
                       sign=np.zeros(c["N"], np.float32))
    return topo.compile(np.asarray(c["counts"], np.float32), pre_sign(c, graded), params, in_scale=in_scale,
                        out_scale=out_scale, sensory_mask=sensory_mask)
