"""fb_lif_step_noalloc, the step for callers that may not allocate device memory: a host
application that hands out every byte of device memory from its own pool, or a real-time control
loop that cannot take the device-wide synchronisation an allocation may imply.

The caller owns every array; the entry point keeps its scratch in a fixed static device array.
These tests play such a caller: they lay a brain out in their own device buffers, step it twice in
a row through the C ABI, and check each result against the ordinary entry point (fb_brains_create
+ fb_step) on the same brain, bit for bit -- the tolerance of every other brain-step test here.
The cases cover conductance- and current-based models, depression, adaptation, background events,
presynaptic inhibition (sequential delivery), non-zero bias and threshold offsets, no drive, a
burst in which every neuron is driven (contributions beyond the in-place buckets), a brain near
the scratch limit, the legacy and a non-blocking stream. This file is collected last and needs no
state from other tests.
"""
import ctypes as C
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("v", "gE", "gI", "refr", "trace", "adapt", "res", "spikeCount")


def _caller_brain(g, p, seed, idx, hz, bias=None, thr=None):
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
    if idx.shape[0]:
        buf["drive"][torch.from_numpy(idx.astype(np.int64)).to(dev)] = torch.from_numpy(
            hz.astype(np.float32)).to(dev)
    if bias is not None:
        buf["bias"].copy_(torch.from_numpy(bias))
    if thr is not None:
        buf["thr"].copy_(torch.from_numpy(thr))
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


def _case(name):
    """(graph, params, seed, driven ids, rates, bias, thr, steps per call) of a named case."""
    from flybrain import SYNTH_PARAMS, synth_graph, workload

    rng = np.random.default_rng(zlib.crc32(name.encode()))
    bias = thr = None
    steps = 400
    if name == "small_workload":  # N=20,000, 1.2M edges: near the scratch limit
        g, idx, hz, _ = workload("small")
        return g, dict(SYNTH_PARAMS), 3, idx.astype(np.int32), np.asarray(hz), None, None, 300
    g = synth_graph(3000, 21)
    idx = rng.choice(g.N, 60, replace=False).astype(np.int32)
    hz = rng.uniform(80, 250, idx.shape[0])
    if name == "coba_dep_bg":
        p = dict(SYNTH_PARAMS, coba=True, adaptInc=0.5, depU=0.1, bgRate=20.0, bgAmp=1.0)
    elif name == "presynaptic_inhibition":
        p = dict(SYNTH_PARAMS, coba=True, preInh=0.5, depU=0.05)
    elif name == "cuba_bias_thr":
        p = dict(SYNTH_PARAMS)
        bias = rng.uniform(-1.0, 4.0, g.N).astype(np.float32)
        thr = rng.uniform(-2.0, 2.0, g.N).astype(np.float32)
    elif name == "no_drive":
        p = dict(SYNTH_PARAMS, bgRate=400.0, bgAmp=5.0)  # background alone drives the network
        idx = np.zeros(0, np.int32)
        hz = np.zeros(0)
    elif name == "every_neuron_driven":
        p = dict(SYNTH_PARAMS, depU=0.02)
        idx = rng.permutation(g.N).astype(np.int32)
        hz = np.full(g.N, 5000.0)  # half the neurons fire at step 0
        steps = 200
    else:
        raise KeyError(name)
    return g, p, 5, idx, hz, bias, thr, steps


CASES = ["coba_dep_bg", "presynaptic_inhibition", "cuba_bias_thr", "no_drive", "every_neuron_driven",
         "small_workload"]


@pytest.mark.parametrize("stream_kind", ["legacy", "non_blocking"])
@pytest.mark.parametrize("name", CASES)
def test_noalloc_step_matches_ordinary_step_twice(name, stream_kind):
    import torch

    from flybrain import LIFCuda
    from flybrain import _native as nat

    L = nat.load()
    g, p, seed, idx, hz, bias, thr, steps = _case(name)
    ref = LIFCuda(g, p, seed=seed)
    for i, h in zip(idx.tolist(), hz.tolist()):
        ref.setDriveOne(int(i), float(h))
    if bias is not None:
        ref.setBias(np.arange(g.N, dtype=np.int32), bias)
    if thr is not None:
        ref.setThrList(np.arange(g.N, dtype=np.int32), thr)
    view, buf = _caller_brain(g, p, seed, idx, hz, bias, thr)
    stream = torch.cuda.Stream() if stream_kind == "non_blocking" else None
    handle = C.c_void_p(stream.cuda_stream) if stream is not None else None

    total = 0
    for call in range(2):
        ref.run(steps)
        rc = L.fb_lif_step_noalloc(C.byref(view), steps, handle)
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
        total += int(buf["spikeCount"].sum().item())
    assert total > 0, "the case produced no spikes"


def test_noalloc_rejects_a_bad_index_and_leaves_the_brain_untouched():
    import torch

    from flybrain import SYNTH_PARAMS, synth_graph
    from flybrain import _native as nat

    L = nat.load()
    g = synth_graph(2000, 4)
    rng = np.random.default_rng(4)
    idx = rng.choice(g.N, 30, replace=False).astype(np.int32)
    hz = np.full(30, 200.0)
    view, buf = _caller_brain(g, dict(SYNTH_PARAMS), 2, idx, hz)
    assert L.fb_lif_step_noalloc(C.byref(view), 50, None) == 0, L.fb_last_error().decode()
    torch.cuda.synchronize()
    before = {k: buf[k].cpu().numpy().copy() for k in FIELDS}
    scal = (view.head, view.rng, view.nFired, view.lastSlot)
    for field, pos, val in (("indices", g.E // 2, g.N), ("driven", 3, -1), ("indptr", 7, g.E + 5)):
        old = buf[field][pos].item()
        buf[field][pos] = val
        torch.cuda.synchronize()
        rc = L.fb_lif_step_noalloc(C.byref(view), 50, None)
        assert rc == nat.FB_EINVAL, field
        assert b"outside" in L.fb_last_error()
        buf[field][pos] = old
        torch.cuda.synchronize()
        for k in FIELDS:
            assert buf[k].cpu().numpy().tobytes() == before[k].tobytes(), (field, k)
        assert (view.head, view.rng, view.nFired, view.lastSlot) == scal
    assert L.fb_lif_step_noalloc(C.byref(view), 50, None) == 0, L.fb_last_error().decode()


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
