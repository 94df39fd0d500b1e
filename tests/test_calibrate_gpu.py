"""The calibrated brain on the device (flybrain/calibrate.py): the compiled weights and signs equal
writeGraph's restatement over the same calibration arrays, and the brain, with its Kenyon-cell
thresholds and lamina biases, steps to the oracle's raster."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tables(tmp_path, N=4000, seed=31):
    from flybrain.connectome import load_connectome, write_connectome
    from flybrain.synth import synth_graph
    g = synth_graph(N, seed)
    rng = np.random.default_rng(seed)
    nt = rng.choice([1, 2, 3, 6, 7], g.N).astype(np.uint8)
    types = [["L1", "L3", "T4a", "OA-VPM3", "KCg", "MN9", "LN"][k] for k in rng.integers(0, 7, g.N)]
    meta = dict(superclasses=["ol_intrinsic", "central", "vnc_intrinsic", "sensory", "descending"],
                classes=["", "Kenyon_Cell", "ALLN"], types=types)
    write_connectome(str(tmp_path), g.N, g.indptr, g.indices, g.counts, nt, min_weight=3, extra=meta)
    c = load_connectome(str(tmp_path))
    c["sc"] = rng.integers(0, 5, g.N).astype(np.uint8)
    c["cls"] = rng.choice([0, 1, 2], g.N, p=[0.8, 0.15, 0.05]).astype(np.uint16)
    size = np.where(rng.random(g.N) < 0.1, 0.0, rng.lognormal(0, 1, g.N)).astype(np.float32)
    return c, size, rng


def test_calibrated_brain_matches_oracle(tmp_path):
    from oracle import oracle as O
    from flybrain.calibrate import create_brain
    from flybrain.connectome import pre_sign
    c, size, rng = _tables(tmp_path)
    opts = dict(coba=True, neuromod=True, wSyn=0.562, sizeAlpha=0.572, kcThreshold=7.319, inhGain=0.577, eInh=-69.079,
                minSyn=6, adaptInc=0.072, tRef=3.682, laminaBias=2.86, dt=0.1, vncGain=1.3,
                typeGain={"T4a": 1.4, "L[13]": 0.8}, classGain={"ALLN": 1.6}, neuronGain=dict(sigma=0.2, seed=5))
    brain, sc = create_brain(c, size, opts, seed=9)
    p = brain.p
    sign = sc["pre_sign"] if sc["pre_sign"] is not None else pre_sign(c)
    W, s = O.write_graph_f64(c["N"], c["indptr"], c["indices"], c["counts"], np.asarray(sign, np.float64), p,
                             in_scale=sc["in_scale"], sensory_mask=sc["sensory_mask"], out_scale=sc["out_scale"])
    w_dev, s_dev = brain.graph.read()
    assert w_dev.tobytes() == W.tobytes() and s_dev.tobytes() == s.tobytes()
    assert (s_dev == 0).sum() > 0                          # octopaminergic neurons silenced

    ob = O.OracleBrain(c["N"], c["indptr"], c["indices"], W, s, p, seed=9)
    kc = np.flatnonzero(c["cls"] == 1)
    for i in kc:
        ob.setThr(int(i), opts["kcThreshold"])
    lam = np.array([i for i, t in enumerate(c["meta"]["types"]) if t in ("L1", "L3")], np.int32)
    ob.setBias(lam, opts["laminaBias"])
    drv = rng.choice(c["N"], 120, replace=False)
    for i in drv:
        brain.setDriveOne(int(i), 180.0)
        ob.setDriveOne(int(i), 180.0)
    brain._batch.record(500, 1 << 20)
    brain.run(500)
    c1, r1 = brain._batch.spike_log(0, 500, 1 << 20)
    c0, r0 = ob.run(500, raster=True)
    assert c0.sum() > 0
    np.testing.assert_array_equal(c1, c0)
    np.testing.assert_array_equal(r1, r0)


def test_graded_sign_and_eye_pairs(tmp_path):
    from oracle import oracle as O
    from flybrain.calibrate import brain_graph
    c, size, rng = _tables(tmp_path, N=1500, seed=32)
    graded = rng.uniform(-1, 1, c["N"]).astype(np.float32)
    eyes = rng.choice(c["N"], 40, replace=False)
    dg, p, sc = brain_graph(c, size, graded, dict(dt=0.1), eye_pairs=eyes)
    assert sc["sensory_mask"][eyes].all() and sc["out_scale"] is None and sc["pre_sign"] is graded
    W, s = O.write_graph_f64(c["N"], c["indptr"], c["indices"], c["counts"], graded.astype(np.float64), p,
                             in_scale=sc["in_scale"], sensory_mask=sc["sensory_mask"])
    w_dev, s_dev = dg.read()
    assert w_dev.tobytes() == W.tobytes() and s_dev.tobytes() == s.tobytes()
