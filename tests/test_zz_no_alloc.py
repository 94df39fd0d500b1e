"""fb_lif_step_noalloc, the step for callers that may not allocate device memory (code inside a
CUDA graph capture, a framework that owns all device memory through its own pool, a real-time
loop that cannot afford an allocation's implicit device synchronisation).

The caller owns every array; the entry point keeps its scratch in a fixed static device array.
This test plays such a caller: it lays a brain out in its own device buffers, steps it twice in a
row through the C ABI, and checks each result against the ordinary entry point (fb_brains_create +
fb_step) on the same brain, bit for bit -- the tolerance of every other brain-step test here.
It lives in a file of its own that pytest collects last, and needs no state from other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("v", "gE", "gI", "refr", "trace", "adapt", "res", "spikeCount")


def _caller_brain(g, p, seed, idx, hz):
    """The brain laid out in caller-owned device memory, as a fresh LIFWasm lays it out."""
    import torch

    from oracle import oracle as O
    from flybrain import _native as nat

    dev = "cuda"
    N = g.N
    ns = O.n_slots(p)
    f32 = lambda: torch.zeros(N, dtype=torch.float32, device=dev)  # noqa: E731
    buf = {k: f32() for k in ("gE", "gI", "refr", "trace", "adapt", "bias", "thr", "drive")}
    buf["v"] = torch.full((N,), float(np.float32(p["vRest"])), dtype=torch.float32, device=dev)
    buf["res"] = torch.ones(N, dtype=torch.float32, device=dev)
    buf["spikeCount"] = torch.zeros(N, dtype=torch.int32, device=dev)
    buf["sign"] = torch.from_numpy(g.sign.copy()).to(dev)
    buf["indptr"] = torch.from_numpy(g.indptr.view(np.int32).copy()).to(dev)
    buf["indices"] = torch.from_numpy(g.indices.view(np.int32).copy()).to(dev)
    buf["weights"] = torch.from_numpy(g.weights.copy()).to(dev)
    buf["ring"] = torch.zeros(ns * N, dtype=torch.int32, device=dev)
    buf["ringCount"] = torch.zeros(ns, dtype=torch.int32, device=dev)
    drv = np.zeros(N, np.int32)
    drv[: idx.shape[0]] = idx
    buf["driven"] = torch.from_numpy(drv).to(dev)
    buf["drive"][torch.from_numpy(idx.astype(np.int64)).to(dev)] = torch.from_numpy(
        hz.astype(np.float32)).to(dev)
    v = nat.FbBrainView()
    v.N, v.nslots, v.head, v.coba = N, ns, 0, 1 if p["coba"] else 0
    names = ("dt", "vRest", "vThresh", "vReset", "tRef", "adaptInc", "depU", "dE", "dTr", "dA",
             "kRec", "kM", "dtS", "eExc", "eInh", "cE", "cI")
    for k, c in zip(names, O.header_constants(p)):
        setattr(v, k, float(c))
    v.rng = O.seed_state(seed)
    for k, t in buf.items():
        setattr(v, k, t.data_ptr())
    v.nDriven = int(idx.shape[0])
    v.nFired = v.lastSlot = 0
    v.bgEvents = float(np.float32(N * p["bgRate"] * p["dt"] / 1000))
    v.bgAmp = float(np.float32(p["bgAmp"]))
    v.bgAcc = 0.0
    v.preInh = float(np.float32(p["preInh"]))
    v.E = g.E
    torch.cuda.synchronize()
    return v, buf


def test_noalloc_step_matches_ordinary_step_twice():
    import torch

    from flybrain import SYNTH_PARAMS, LIFCuda, synth_graph
    from flybrain import _native as nat

    L = nat.load()
    g = synth_graph(3000, 21)
    rng = np.random.default_rng(21)
    idx = rng.choice(g.N, 60, replace=False).astype(np.int32)
    hz = rng.uniform(80, 250, idx.shape[0])
    p = dict(SYNTH_PARAMS, adaptInc=0.5, depU=0.1, bgRate=20.0, bgAmp=1.0)

    ref = LIFCuda(g, p, seed=5)
    for i, h in zip(idx, hz):
        ref.setDriveOne(int(i), float(h))
    view, buf = _caller_brain(g, p, 5, idx, hz)

    for call in range(2):
        ref.run(400)
        rc = L.fb_lif_step_noalloc(C.byref(view), 400, None)
        assert rc == 0, L.fb_last_error().decode()
        torch.cuda.synchronize()
        for k in FIELDS:
            got = buf[k].cpu().numpy()
            want = getattr(ref, k)
            assert got.tobytes() == want.tobytes(), (call, k)
        sc = ref._batch.scalars(0)
        assert view.nFired == sc["nFired"] and view.lastSlot == sc["lastSlot"], call
        assert view.rng == sc["rng"] and view.head == sc["head"], call
        fired = buf["ring"][view.lastSlot * g.N: view.lastSlot * g.N + view.nFired].cpu().numpy()
        np.testing.assert_array_equal(fired, ref._batch.fired(0))


def test_noalloc_rejects_a_brain_larger_than_its_scratch():
    from flybrain import _native as nat

    L = nat.load()
    v = nat.FbBrainView()
    v.N, v.nslots, v.head, v.E = 165122, 19, 0, 11_000_000
    for k in ("v", "gE", "gI", "refr", "trace", "adapt", "res", "bias", "thr", "drive", "sign",
              "spikeCount", "indptr", "indices", "weights", "ring", "ringCount", "driven"):
        setattr(v, k, 256)  # never dereferenced: the size check comes first
    rc = L.fb_lif_step_noalloc(C.byref(v), 1, None)
    assert rc == nat.FB_EINVAL
    assert b"scratch" in L.fb_last_error()
