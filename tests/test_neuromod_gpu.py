"""The calibrated brain with neuromodulation in closed loop on the device: the controller
(flybrain/neuromod.py) drives a LIFCuda brain and, separately, the oracle brain on the same
tables, millisecond by millisecond (10 brain steps per millisecond, the controller's conductances,
rate filter, threshold or gain field in between). Rasters, thresholds, signs and the controller's
own state agree bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tables(tmp_path, N=3000, seed=41):
    from flybrain.connectome import load_connectome, write_connectome
    from flybrain.synth import synth_graph
    g = synth_graph(N, seed)
    rng = np.random.default_rng(seed)
    nt = rng.choice([1, 2, 3, 6], g.N).astype(np.uint8)
    kinds = ["L1", "T4a", "OA-VUMa2", "OA-AL2i3", "OA-VPM4", "IPC", "KCg", "MN9", "LN"]
    types = [kinds[k] for k in rng.choice(len(kinds), g.N, p=[.1, .2, .02, .02, .02, .01, .13, .2, .3])]
    meta = dict(superclasses=["ol_intrinsic", "central", "vnc_intrinsic", "sensory", "descending"],
                classes=["", "Kenyon_Cell"], types=types)
    write_connectome(str(tmp_path), g.N, g.indptr, g.indices, g.counts, nt, min_weight=3, extra=meta)
    c = load_connectome(str(tmp_path))
    c["sc"] = rng.integers(0, 5, g.N).astype(np.uint8)
    c["cls"] = np.array([1 if t == "KCg" else 0 for t in types], np.uint16)
    size = rng.lognormal(0, 1, g.N).astype(np.float32)
    return c, size, rng


@pytest.mark.parametrize("mode", ["thrField", "gainField"])
def test_closed_loop_matches_the_oracle(tmp_path, mode):
    from oracle import oracle as O
    from flybrain.calibrate import create_brain
    from flybrain.connectome import pre_sign
    from flybrain.neuromod import Neuromod
    c, size, rng = _tables(tmp_path)
    opts = dict(coba=True, neuromod=True, wSyn=0.562, sizeAlpha=0.572, kcThreshold=7.319, inhGain=0.577,
                eInh=-69.079, minSyn=6, adaptInc=0.072, tRef=3.682, laminaBias=2.86, dt=0.1)
    brain, sc = create_brain(c, size, opts, seed=5)
    p = brain.p
    sign = sc["pre_sign"] if sc["pre_sign"] is not None else pre_sign(c)
    W, s = O.write_graph_f64(c["N"], c["indptr"], c["indices"], c["counts"], np.asarray(sign, np.float64), p,
                             in_scale=sc["in_scale"], sensory_mask=sc["sensory_mask"], out_scale=sc["out_scale"])
    s0 = s.copy()  # the oracle brain writes its sign array in place under gainField
    ob = O.OracleBrain(c["N"], c["indptr"], c["indices"], W, s, p, seed=5)
    for i in np.flatnonzero(c["cls"] == 1):
        ob.setThr(int(i), opts["kcThreshold"])
    ob.setBias(np.array([i for i, t in enumerate(c["meta"]["types"]) if t == "L1"], np.int32), opts["laminaBias"])
    drv = rng.choice(c["N"], 150, replace=False)
    for i in drv:
        brain.setDriveOne(int(i), 160.0)
        ob.setDriveOne(int(i), 160.0)
    params = dict(oaMode=mode)
    if mode == "gainField":
        params["oaTargets"] = dict(gainField=dict(superclasses=["ol_intrinsic"], types=["MN9"]))
    calib = dict(oaThr={str(i): 3.0 for i in range(0, c["N"], 97)}, ipcThr={})
    nm_gpu = Neuromod(c, brain, calib=calib, min_syn=6, params=params)
    nm_ref = Neuromod(c, ob, calib=calib, min_syn=6, params=params)
    ms, per_ms = 160, 10
    brain._batch.record(ms * per_ms, 1 << 20)
    counts, raster = [], []
    for t in range(ms):
        sugar = 0.9 - 0.8 * t / ms  # the fly starves: AKH rises, IPC drive falls
        brain.run(per_ms)
        k, r = ob.run(per_ms, raster=True)
        counts.append(k)
        raster.append(r)
        nm_gpu.update(1, sugar, 0.5)
        nm_ref.update(1, sugar, 0.5)
    c1, r1 = brain._batch.spike_log(0, ms * per_ms, 1 << 20)
    c0, r0 = np.concatenate(counts), np.concatenate(raster)
    assert c0.sum() > 0 and len(nm_gpu.targets) > 0
    np.testing.assert_array_equal(c1, c0)
    np.testing.assert_array_equal(r1, r0)
    assert brain._batch.read("thr", 0).tobytes() == ob.thr.tobytes()
    assert brain.graph.read()[1].tobytes() == ob.sign.tobytes()
    for k in ("r", "x", "shift", "base"):
        assert getattr(nm_gpu, k).tobytes() == getattr(nm_ref, k).tobytes(), k
    assert (nm_gpu.akh, nm_gpu.dilp) == (nm_ref.akh, nm_ref.dilp)
    if mode == "thrField":
        assert (nm_gpu.shift > 0).any()
    else:
        assert (brain.graph.read()[1] != s0).any()
