"""The flyvis oracle (oracle/lifsim.c ob_fv_run, a restatement of lif.c's fv_step) against the
reference's own fv_step: the committed golden run (tests/golden/flyvis/flyvis_synth.npz, made by
tests/golden/make_golden.py from the reference build) and, where the reference tree is present,
a fresh comparison; plus the export format and the synthetic model's shape."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O


def _golden():
    z = np.load(os.path.join(GOLDEN, "flyvis", "flyvis_synth.npz"))
    m = dict(N=int(z["N"]), E=int(z["E"]), indptr=z["indptr"], target=z["target"], weight=z["weight"],
             bias=z["bias"], tau=z["tau"], dt=float(z["dt"]))
    return m, z


def test_oracle_matches_the_reference_golden_run():
    from oracle import oracle as O
    m, z = _golden()
    v = np.tile(m["bias"], (z["x"].shape[0], 1)).astype(np.float32)
    done = 0
    for k, upto in enumerate(z["steps"]):
        O.fv_run(m, v, z["x"].copy(), int(upto) - done)
        done = int(upto)
        assert v.tobytes() == z["v"][k].tobytes(), int(upto)
    assert np.isfinite(v).all() and (v < 0).any() and (v > 0).any()


@pytest.mark.skipif(not O.have_reference_build(), reason="reference kernel not built here")
def test_oracle_matches_the_reference_fv_step():
    from oracle import oracle as O
    from flybrain.flyvis import synth_flyvis
    m = synth_flyvis(N=63 * 30, seed=9, columns=30)
    rng = np.random.default_rng(9)
    x = rng.normal(0, 1, (2, m["N"])).astype(np.float32)
    a = np.tile(m["bias"], (2, 1)).astype(np.float32)
    b = a.copy()
    O.fv_run(m, a, x, 60, backend="port")
    O.fv_run(m, b, x, 60, backend="ref")
    assert a.tobytes() == b.tobytes()


def test_export_format_round_trip():
    from flybrain.flyvis import flyvis_bytes, parse_flyvis, synth_flyvis
    m = synth_flyvis(N=63 * 4, seed=2, columns=4)
    buf = flyvis_bytes(m)
    assert len(buf) == m["N"] * (1 + 2 + 2 + 4 + 4) + (m["N"] + 1) * 4 + m["E"] * 8
    p = parse_flyvis(buf, dict(N=m["N"], E=m["E"], types=m["types"]), m["inputIdx"])
    for k in ("tid", "u", "v", "bias", "tau", "indptr", "target", "weight"):
        np.testing.assert_array_equal(p[k], m[k])
    with pytest.raises(ValueError):
        parse_flyvis(buf[:-4], dict(N=m["N"], E=m["E"]))


def test_synthetic_model_has_the_reference_shape():
    """45,669 nodes and about 1.5 M synapses per eye with a median of 33 incoming edges
    (src/flyvisgpu.js:3-5, :24-25); the fixture is the same recipe at 630 nodes."""
    from flybrain.flyvis import synth_flyvis
    m = synth_flyvis()
    assert m["N"] == 45669 and 1.4e6 < m["E"] < 1.6e6
    assert np.median(np.bincount(m["target"], minlength=m["N"])) == 33
    assert all(ix.shape[0] == 721 for ix in m["inputIdx"].values())
    g, z = _golden()
    s = synth_flyvis(N=630, seed=5, columns=10)
    for k in ("indptr", "target", "weight", "bias", "tau"):
        np.testing.assert_array_equal(s[k], g[k])
