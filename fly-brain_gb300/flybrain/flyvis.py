"""The flyvis optic lobe on the GB300 kernels: a drop-in for the reference's FlyVis
(src/flyvis.js: one instance per eye running lif.c's fv_step, src/wasm/lif.c:82-93), here a batch
of B eyes sharing one model and stepped together (fb_flyvis_*).

  FlyVis(model, B=1)       model as parse_flyvis returns it (N, E, indptr, target, weight, bias,
                           tau, inputIdx, dt); instance 0 is the reference's single eye
  .setInput(lum, b=0)      luminance per hex column into every input type's nodes
  .step(n=1) / .reset(b)   fv_step for every instance / v = bias
  .v(b) / .read / .write   instance b's activity (or input)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat

FV_V, FV_X = 0, 1


def kdt_of(tau, dt):
    """dt / max(tau, dt) in double, stored f32 (src/flyvis.js:13)."""
    tau = np.asarray(tau, np.float64)
    return (dt / np.maximum(tau, dt)).astype(np.float32)


def parse_flyvis(buf: bytes, meta: dict, inputs: dict | None = None) -> dict:
    """The reference's flyvis export (parseFlyVis, src/flyvis.js:25-31): tid u8[N], u i16[N],
    v i16[N], bias f32[N], tau f32[N], indptr i32[N+1], target i32[E], weight f32[E], packed
    in that order with no padding; N, E and the type names from the JSON side."""
    N, E = int(meta["N"]), int(meta["E"])
    b = np.frombuffer(buf, dtype=np.uint8)
    o = 0

    def take(dt, n):
        nonlocal o
        nb = n * np.dtype(dt).itemsize
        if o + nb > b.shape[0]:
            raise ValueError(f"flyvis export truncated: need {o + nb} bytes, have {b.shape[0]}")
        a = b[o:o + nb].copy().view(dt)
        o += nb
        return a
    tid, u, v = take(np.uint8, N), take(np.int16, N), take(np.int16, N)
    bias, tau = take(np.float32, N), take(np.float32, N)
    indptr, target, weight = take(np.int32, N + 1), take(np.int32, E), take(np.float32, E)
    return dict(N=N, E=E, tid=tid, u=u, v=v, bias=bias, tau=tau, indptr=indptr, target=target, weight=weight,
                types=meta.get("types"), inputIdx=inputs or {}, dt=0.02)


def flyvis_bytes(model: dict) -> bytes:
    """The inverse of parse_flyvis (the export's binary layout)."""
    parts = [np.asarray(model["tid"], np.uint8), np.asarray(model["u"], np.int16), np.asarray(model["v"], np.int16),
             np.asarray(model["bias"], np.float32), np.asarray(model["tau"], np.float32),
             np.asarray(model["indptr"], np.int32), np.asarray(model["target"], np.int32),
             np.asarray(model["weight"], np.float32)]
    return b"".join(np.ascontiguousarray(p).tobytes() for p in parts)


def synth_flyvis(N: int = 45669, seed: int = 1, mean_in: float = 33.0, columns: int = 721,
                 n_types: int = 63) -> dict:
    """Seeded flyvis-shaped model (a stand-in for the reference's export, which is not in the
    tree): N nodes of n_types cell types over `columns` hex columns, Poisson(mean_in) outgoing
    edges per node to targets in nearby columns (75%) or anywhere (25%), weights sign x
    lognormal(-3, 0.7) with one sign per source type, bias N(0, 0.5), tau U(0.02, 0.2) s,
    dt 0.02 s; R1-R8 input nodes are the first 8 types' nodes, one per column."""
    rng = np.random.default_rng(seed)
    tid = (np.arange(N) % n_types).astype(np.uint8)
    col = (np.arange(N) // n_types) % columns
    deg = rng.poisson(mean_in, N).astype(np.int64)
    src = np.repeat(np.arange(N, dtype=np.int64), deg)
    E = int(src.shape[0])
    local = rng.random(E) < 0.75
    near_col = (col[src] + rng.integers(-6, 7, E)) % columns
    near = near_col * n_types + rng.integers(0, n_types, E)
    near = np.where(near < N, near, rng.integers(0, N, E))
    tgt = np.where(local, near, rng.integers(0, N, E)).astype(np.int32)
    type_sign = np.where(rng.random(n_types) < 0.55, 1.0, -1.0)
    w = (type_sign[tid[src]] * rng.lognormal(-3.0, 0.7, E)).astype(np.float32)
    indptr = np.zeros(N + 1, np.int32)
    np.cumsum(deg, out=indptr[1:])
    inputs = {f"R{k + 1}": np.nonzero(tid == k)[0][:columns].astype(np.int32) for k in range(8)}
    return dict(N=N, E=E, tid=tid, u=(col % 64).astype(np.int16), v=(col // 64).astype(np.int16),
                bias=rng.normal(0.0, 0.5, N).astype(np.float32),
                tau=rng.uniform(0.02, 0.2, N).astype(np.float32), indptr=indptr, target=tgt, weight=w,
                types=[f"T{k}" for k in range(n_types)], inputIdx=inputs, dt=0.02)


class FlyVis:
    """B eyes sharing one flyvis model on the device (src/flyvis.js's FlyVis, batched)."""

    def __init__(self, model: dict, B: int = 1):
        self.L = nat.load()
        self.model = model
        self.N, self.E, self.B = int(model["N"]), int(model["E"]), int(B)
        self.dt = float(model.get("dt") or 0.02)
        self.inputIdx = {k: np.ascontiguousarray(v, np.int32) for k, v in (model.get("inputIdx") or {}).items()}
        kdt = model["kdt"] if model.get("kdt") is not None else kdt_of(model["tau"], self.dt)
        self._keep = [np.ascontiguousarray(model["indptr"], np.int32), np.ascontiguousarray(model["target"], np.int32),
                      np.ascontiguousarray(model["weight"], np.float32), np.ascontiguousarray(model["bias"], np.float32),
                      np.ascontiguousarray(kdt, np.float32)]
        ip, tg, w, bias, k = self._keep
        h = C.c_void_p()
        nat.check(self.L.fb_flyvis_create(self.N, self.E, nat.ptr(ip), nat.ptr(tg), nat.ptr(w), nat.ptr(bias),
                                          nat.ptr(k), self.B, C.byref(h)))
        self.h = h
        self._idx = None

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.fb_flyvis_destroy(h)
            self.h = None

    def setInput(self, lum, b: int = 0):
        """lum: luminance per hex column, the same for every input type (src/flyvis.js:20-21)."""
        if self._idx is None:
            idx = [self.inputIdx[t] for t in self.inputIdx]
            self._idx = (np.concatenate(idx) if idx else np.zeros(0, np.int32),
                         [ix.shape[0] for ix in idx])
        lum = np.asarray(lum, np.float32)
        vals = np.concatenate([lum[:n] for n in self._idx[1]]) if self._idx[1] else np.zeros(0, np.float32)
        self.set_input(self._idx[0], vals, b)

    def set_input(self, idx, values, b: int = 0):
        idx = np.ascontiguousarray(idx, np.int32)
        values = np.ascontiguousarray(values, np.float32)
        nat.check(self.L.fb_flyvis_set_input(self.h, int(b), idx.shape[0], nat.ptr(idx), nat.ptr(values)))

    def step(self, n: int = 1):
        nat.check(self.L.fb_flyvis_step(self.h, int(n)))

    def reset(self, b: int = -1):
        nat.check(self.L.fb_flyvis_reset(self.h, int(b)))

    def read(self, field: str = "v", b: int = 0) -> np.ndarray:
        out = np.zeros(self.N, np.float32)
        nat.check(self.L.fb_flyvis_read(self.h, FV_V if field == "v" else FV_X, int(b), nat.ptr(out)))
        return out

    def write(self, field: str, b: int, values):
        a = np.ascontiguousarray(values, np.float32)
        nat.check(self.L.fb_flyvis_write(self.h, FV_V if field == "v" else FV_X, int(b), nat.ptr(a)))

    def v(self, b: int = 0) -> np.ndarray:
        return self.read("v", b)

    def last_ms(self) -> float:
        ms = C.c_float()
        nat.check(self.L.fb_flyvis_last_ms(self.h, C.byref(ms)))
        return ms.value
