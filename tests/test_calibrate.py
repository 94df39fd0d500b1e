"""Host side of the calibrated brain (flybrain/calibrate.py, after src/brainmodel.js:7-100 and
src/ratenet.js:22-31): region medians, size scales, sensory mask, class physiology, modulatory sign
and type gains on hand-worked tables; the real data directory's tables when present.

No JavaScript engine is available to run the reference's functions, so these values are pinned by
hand-worked cases and by the reference's formulas, not by the reference's own output."""
import math
import os

import numpy as np
import pytest

from refpaths import REF_DATA


def _tables():
    """Nine neurons over five superclasses (regions 0, 1, 2, 1, 2), three classes, a few types."""
    meta = dict(superclasses=["ol_intrinsic", "central", "vnc_intrinsic", "sensory", "descending"],
                classes=["", "Kenyon_Cell", "ALLN"],
                types=["L1", "L6", "OA-VPM3", "KCab", "T4a", "L5", "OA-AL2i1", "MN9", "L12"])
    sc = np.array([0, 0, 1, 1, 2, 0, 3, 4, 1], np.uint8)
    cls = np.array([0, 0, 0, 1, 0, 0, 2, 0, 1], np.uint16)
    nt = np.array([1, 2, 6, 1, 3, 7, 6, 1, 2], np.uint8)
    size = np.array([4.0, 1.0, 10.0, 0.0, 8.0, 2.0, 6.0, 2.0, 30.0], np.float32)
    return dict(N=9, meta=meta, sc=sc, cls=cls, nt=nt), size


def test_region_medians_and_reference_volume():
    from flybrain.calibrate import region_of, region_size_ref
    c, size = _tables()
    assert [region_of(n) for n in c["meta"]["superclasses"]] == [0, 1, 2, 1, 2]
    assert region_of("visual_projection") == 0 and region_of("sensory_ascending") == 2 and region_of(None) == 1
    ref, med, region = region_size_ref(c["meta"]["superclasses"], c["sc"], size)
    np.testing.assert_array_equal(region, [0, 0, 1, 1, 2, 0, 1, 2, 1])
    # region 0 sizes {4, 1, 2} -> sorted [1, 2, 4], index 1 -> 2; region 1 {10, 0, 6, 30} -> [6, 10, 30] -> 10;
    # region 2 {8, 2} -> [2, 8], index 1 -> 8
    assert med == [2.0, 10.0, 8.0]
    np.testing.assert_array_equal(ref, np.array([2, 2, 10, 10, 8, 2, 10, 8, 10], np.float32))
    _, med, _ = region_size_ref(c["meta"]["superclasses"], c["sc"], np.zeros(9, np.float32))
    assert med == [1.0, 1.0, 1.0]


def test_size_scales_and_sensory_mask():
    from flybrain.calibrate import brain_scales
    c, size = _tables()
    o = dict(sizeAlpha=0.5, maxSizeScale=20.0, boostCap=1.5, vncGain=1.25)
    in_scale, mask, region = brain_scales(c, size, o)
    ref = [2, 2, 10, 10, 8, 2, 10, 8, 10]
    for i in range(9):
        s = min(20.0, max(1 / 20.0, float(size[i]) / ref[i])) if size[i] > 0 else 1.0
        want = min(1.5, s ** -0.5) * (1.25 if region[i] == 2 else 1.0)
        assert in_scale[i] == np.float32(want), i
    # neuron 1: size 1 / median 2 -> 0.5^-0.5 = 1.414 (under the cap); neuron 8: 30/10 -> 3^-0.5
    assert in_scale[1] == np.float32(math.sqrt(2.0)) and in_scale[8] == np.float32(3.0 ** -0.5)
    assert in_scale[3] == np.float32(1.0)                    # unknown size: s = 1
    np.testing.assert_array_equal(mask, [0, 0, 0, 0, 0, 0, 1, 0, 0])
    in_scale, _, _ = brain_scales(c, size, dict(boostCap=1.0))
    assert in_scale.max() <= 1.0
    tiny = dict(c, N=3, sc=np.array([1, 1, 1], np.uint8))
    s3, _, _ = brain_scales(tiny, np.array([1e-6, 1, 1e6], np.float32), dict(boostCap=10.0))
    np.testing.assert_array_equal(s3, np.float32([20.0 ** 0.5, 1.0, 20.0 ** -0.5]))   # s clamped to 1/20 and 20


def test_class_physiology_selects_kenyon_and_lamina_cells():
    from flybrain.calibrate import class_physiology
    c, _ = _tables()
    (kc, kv), (lam, lv) = class_physiology(c, dict(kcThreshold=7.319, laminaBias=2.86))
    np.testing.assert_array_equal(kc, [3, 8])
    np.testing.assert_array_equal(lam, [0, 5])               # L1, L5; not L6 or L12
    assert (kv, lv) == (7.319, 2.86)


def test_modulatory_sign():
    from flybrain.calibrate import modulatory_sign
    from flybrain.connectome import EXC_SIGN
    c, _ = _tables()
    assert modulatory_sign(c, None, {}) is None
    given = np.linspace(-1, 1, 9).astype(np.float32)
    assert modulatory_sign(c, given, {}) is given
    s = modulatory_sign(c, None, dict(neuromod=True))
    want = EXC_SIGN[c["nt"]].copy()
    want[[2, 6]] = 0
    np.testing.assert_array_equal(s, want)
    s = modulatory_sign(c, given, dict(neuromod=True))
    assert s[2] == 0 and s[6] == 0 and s[0] == given[0] and given[2] != 0
    np.testing.assert_array_equal(modulatory_sign(c, None, dict(neuromod=True, oaMode="synFast")), EXC_SIGN[c["nt"]])


def test_type_gains_exact_regex_class_and_table():
    from flybrain.calibrate import type_gains
    c, _ = _tables()
    assert type_gains(c, {}) is None
    assert type_gains(c, dict(typeGain={"L1": 1}, classGain={"ALLN": 1})) is None
    g = type_gains(c, dict(typeGain={"L1": 1.3, "OA-.*": 0.7, "T4a|MN9": 2.0}, classGain={"Kenyon_Cell": 0.9},
                           neuronGainTable={"4": 0.5}))
    f = np.float32
    want = [f(1.3), f(1), f(0.7), f(0.9), f(f(2.0) * math.exp(0.5)), f(1), f(0.7), f(2.0), f(0.9)]
    np.testing.assert_array_equal(g, np.array(want, np.float32))
    # "L1" is an exact name (no regular-expression character), so "L12" is not matched
    assert g[8] == f(0.9)
    tab = np.array([0, 0.1, np.nan, 0, 0, 0, 0, 0, -0.2])
    g = type_gains(c, dict(neuronGainTable=tab))
    np.testing.assert_array_equal(g, np.float32([1, math.exp(0.1), 1, 1, 1, 1, 1, 1, math.exp(-0.2)]))


def test_type_gains_round_to_float32_after_every_multiply():
    from flybrain.calibrate import type_gains
    c, _ = _tables()
    a, b = 1.0000001, 1.00000007
    g = type_gains(c, dict(typeGain={"L1": a}, classGain={"": b}))
    step = np.float32(np.float32(a) * b)          # the reference stores a Float32Array between the two
    assert g[0] == step
    assert g[0] == np.float32(float(np.float32(a)) * b)


def test_lognormal_individual():
    from flybrain.calibrate import type_gains
    N = 20000
    c = dict(N=N, meta=dict(types=[""] * N, classes=[""]), cls=np.zeros(N, np.uint16))
    g1 = type_gains(c, dict(neuronGain=dict(sigma=0.3, seed=7)))
    g2 = type_gains(c, dict(neuronGain=dict(sigma=0.3, seed=7)))
    g3 = type_gains(c, dict(neuronGain=dict(sigma=0.3, seed=8)))
    assert g1.tobytes() == g2.tobytes() and g1.tobytes() != g3.tobytes()
    lg = np.log(g1.astype(np.float64))
    assert abs(lg.mean()) < 0.01 and abs(lg.std() - 0.3) < 0.01
    assert (g1 > 0).all()


def test_mulberry32_stream():
    """The generator's first words, computed with explicit 32-bit wrap-around steps."""
    from flybrain.calibrate import _mulberry32_lognormal
    M = 0xFFFFFFFF

    def words(seed, n):
        a = int(math.fmod(float(seed) * 2654435761.0, 4294967296.0))  # JS: the product in double
        out = []
        for _ in range(n):
            a = (a + 0x6D2B79F5) & M
            t = ((a ^ (a >> 15)) * (a | 1)) & M
            t2 = ((t ^ (t >> 7)) * (t | 61)) & M
            t = ((t + t2) & M) ^ t
            out.append((t ^ (t >> 14)) / 2.0 ** 32)
        return out
    u = words(1, 4)
    want = [math.exp(0.5 * math.sqrt(-2 * math.log(u[0])) * math.cos(2 * math.pi * u[1])),
            math.exp(0.5 * math.sqrt(-2 * math.log(u[2])) * math.cos(2 * math.pi * u[3]))]
    np.testing.assert_array_equal(_mulberry32_lognormal(2, 0.5, 1), np.array(want))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DATA, "meta.json")), reason="no connectome data directory")
def test_real_tables_calibrate():
    """The reference's data directory and parameter set: every scale finite and in range, the
    named populations present."""
    import json
    from flybrain.calibrate import brain_scales, class_physiology, modulatory_sign
    from flybrain.connectome import load_connectome
    c = load_connectome(REF_DATA)
    o = json.load(open(os.path.join(REF_DATA, "brain_params.json")))
    in_scale, mask, region = brain_scales(c, c["size"], o)
    assert np.isfinite(in_scale).all() and in_scale.max() <= 1.0 and in_scale.min() >= 20.0 ** -o["sizeAlpha"] - 1e-6
    assert 0 < mask.sum() < c["N"] and set(np.unique(region)) == {0, 1, 2}
    (kc, _), (lam, _) = class_physiology(c, o)
    assert kc.shape[0] > 1000 and lam.shape[0] > 100
    s = modulatory_sign(c, c["ntsign"], o)
    assert (s == 0).sum() > (np.asarray(c["ntsign"]) == 0).sum()
