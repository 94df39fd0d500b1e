"""Test helper: a pure-Python FLYG / FLYN encoder (src/codec/rc.js Encoder and UInt.code,
src/codec/graph.js:16-67 encodeGraph, src/codec/neurons.js:11-23 encodeNeurons), used to make
streams for the native decoders from synthetic tables. Small inputs only."""
from __future__ import annotations

import numpy as np

TOP = 1 << 24
ONE = 1 << 12


def lg(x: int) -> int:
    """Bit length of x + 1 less one (src/codec/rc.js:125)."""
    return (int(x) + 1).bit_length() - 1


class Encoder:
    """LZMA-style carry-less range encoder, 12-bit probabilities (src/codec/rc.js:6-29)."""

    def __init__(self):
        self.out = bytearray()
        self.low = 0
        self.range = 0xFFFFFFFF
        self.cache = 0
        self.cache_size = 1

    def _shift_low(self):
        if self.low < 0xFF000000 or self.low >= 1 << 32:
            carry = 1 if self.low >= 1 << 32 else 0
            t = self.cache
            while True:
                self.out.append((t + carry) & 0xFF)
                t = 0xFF
                self.cache_size -= 1
                if self.cache_size == 0:
                    break
            self.cache = (self.low >> 24) & 0xFF
        self.cache_size += 1
        self.low = (self.low % TOP) * 256

    def _norm(self):
        while self.range < TOP:
            self.range = (self.range * 256) & 0xFFFFFFFF
            self._shift_low()

    def bit(self, p, i, b):
        pr = int(p[i])
        bound = (self.range >> 12) * pr
        if b == 0:
            self.range = bound
            p[i] = pr + ((ONE - pr) >> 5)
        else:
            self.low += bound
            self.range -= bound
            p[i] = pr - (pr >> 5)
        self._norm()
        return b

    def direct(self, v, nbits):
        while nbits > 0:
            n = min(nbits, 16)
            nbits -= n
            self.range >>= n
            self.low += ((v >> nbits) % (1 << n)) * self.range
            self._norm()

    def finish(self) -> bytes:
        for _ in range(5):
            self._shift_low()
        return bytes(self.out)


def probs(n):
    return np.full(n, ONE >> 1, np.int64)


class UInt:
    """Adaptive Elias-gamma model (src/codec/rc.js:79-97), encoding side."""

    def __init__(self, nctx):
        self.k = probs(nctx * 32)
        self.m = probs(nctx * 32 * 4)

    def code(self, e: Encoder, ctx: int, v: int):
        n = int(v) + 1
        kk = n.bit_length() - 1
        base = ctx * 32
        t = 1
        for i in range(4, -1, -1):
            t = (t << 1) | e.bit(self.k, base + t, (kk >> i) & 1)
        k = t - 32
        if k == 0:
            return
        mb = (base + k) * 4
        b1 = e.bit(self.m, mb + 1, (n >> (k - 1)) & 1)
        if k >= 2:
            e.bit(self.m, mb + 2 + b1, (n >> (k - 2)) & 1)
        if k >= 3:
            rest = k - 2
            e.direct(n & ((1 << rest) - 1), rest)


class SInt(UInt):
    def code(self, e, ctx, v):
        super().code(e, ctx, 2 * v if v >= 0 else -2 * v - 1)


def encode_flyg(N, indptr, indices, weights, min_weight, order=None) -> bytes:
    """graph.js encodeGraph: rows in `order` (new -> old id), copy bits over the previous row,
    residual targets as a first offset and gaps, weights context-modelled."""
    order = np.arange(N) if order is None else np.asarray(order)
    inv = np.zeros(N, np.int64)
    inv[order] = np.arange(N)
    E = int(indptr[N])
    e = Encoder()
    deg_m, first_m, gap_m, w_m, copy_m = UInt(24), SInt(24), UInt(24), UInt(48), probs(64)
    for r in range(N):
        e.direct(int(order[r]), 18)
    prevT, prevW, prevDeg = [], [], 0
    for r in range(N):
        o = int(order[r])
        a, b = int(indptr[o]), int(indptr[o + 1])
        d = b - a
        row = sorted((int(inv[indices[k]]), int(weights[k])) for k in range(a, b))
        deg_m.code(e, min(lg(prevDeg), 23), d)
        ratio = min(7, max(0, lg(d) - lg(len(prevT)) + 4)) if prevT else 0
        tset = {t for t, _ in row}
        in_prev = {}
        pb = 0
        for i, t in enumerate(prevT):
            hit = 1 if t in tset else 0
            e.bit(copy_m, (pb * 8 + ratio) * 2 + (1 if i == 0 else 0), hit)
            pb = hit
            if hit:
                in_prev[t] = prevW[i]
        last, pg, first = -1, 0, True
        for t, _ in row:
            if t in in_prev:
                continue
            if first:
                first_m.code(e, min(lg(d), 23), t - r)
                first = False
            else:
                g = t - last - 1
                gap_m.code(e, min(lg(pg), 23), g)
                pg = g
            last = t
        pw = 0
        for t, w in row:
            ref = in_prev.get(t)
            ctx = 24 + min(lg(ref - min_weight), 23) if ref is not None else min(lg(pw), 23)
            w_m.code(e, ctx, w - min_weight)
            pw = w - min_weight
        prevT = [t for t, _ in row]
        prevW = [w for _, w in row]
        prevDeg = d
    head = np.array([0x47594C46, 1, N, E, min_weight], np.uint32).tobytes()
    return head + e.finish()


def encode_flyn(body_ids, soma, cls, nt, superclass, side) -> bytes:
    """neurons.js encodeNeurons: body-id gaps, superclass then class / transmitter / side in its
    context, a has-soma bit, soma offsets (integer voxels)."""
    N = len(body_ids)
    e = Encoder()
    id_m, sc_m, cls_m, nt_m, side_m, has_m, soma_m = UInt(1), UInt(32), UInt(32), UInt(32), UInt(32), probs(2), SInt(3)
    prev_id, prev, ph = 0, [0, 0, 0], 1
    for i in range(N):
        bid = int(body_ids[i])
        id_m.code(e, 0, bid - prev_id)
        prev_id = bid
        s = int(superclass[i])
        sc_m.code(e, 0, s)
        cls_m.code(e, s, int(cls[i]))
        nt_m.code(e, s, int(nt[i]))
        side_m.code(e, s, int(side[i]))
        has = 1 if np.isfinite(soma[i][0]) else 0
        e.bit(has_m, ph, has)
        ph = has
        if has:
            for k in range(3):
                soma_m.code(e, k, int(soma[i][k]) - prev[k])
                prev[k] = int(soma[i][k])
    head = np.array([0x4E594C46, 1, N], np.uint32).tobytes()
    return head + e.finish()
