"""The flyvis kernel (fb_flyvis_*, fly-brain_gb300/csrc/fb_flyvis.cu) against the reference's
fv_step: the golden run bit for bit, full-size eyes against the oracle, input semantics."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _golden():
    z = np.load(os.path.join(GOLDEN, "flyvis", "flyvis_synth.npz"))
    m = dict(N=int(z["N"]), E=int(z["E"]), indptr=z["indptr"], target=z["target"], weight=z["weight"],
             bias=z["bias"], tau=z["tau"], dt=float(z["dt"]))
    return m, z


def test_golden_run_bit_for_bit():
    from flybrain.flyvis import FlyVis
    m, z = _golden()
    B = z["x"].shape[0]
    fv = FlyVis(m, B=B)
    for b in range(B):
        fv.write("x", b, z["x"][b])
        np.testing.assert_array_equal(fv.v(b), m["bias"])
    done = 0
    for k, upto in enumerate(z["steps"]):
        fv.step(int(upto) - done)
        done = int(upto)
        for b in range(B):
            assert fv.v(b).tobytes() == z["v"][k][b].tobytes(), (int(upto), b)


@pytest.mark.parametrize("B", [1, 2, 5, 33, 64])
def test_full_size_eyes_match_the_oracle(B):
    from oracle import oracle as O
    from flybrain.flyvis import FlyVis, synth_flyvis
    m = synth_flyvis(seed=7)
    rng = np.random.default_rng(B)
    x = rng.normal(0.2, 0.6, (B, m["N"])).astype(np.float32)
    fv = FlyVis(m, B=B)
    for b in range(B):
        fv.write("x", b, x[b])
    fv.step(25)
    v = np.tile(m["bias"], (B, 1)).astype(np.float32)
    O.fv_run(m, v, x, 25)
    for b in range(B):
        assert fv.v(b).tobytes() == v[b].tobytes(), b


def test_set_input_and_reset():
    """setInput writes luminance into every input type's nodes, per column (src/flyvis.js:20-21);
    a repeated index keeps its last value; reset puts v back to bias for one eye."""
    from flybrain.flyvis import FlyVis, synth_flyvis
    m = synth_flyvis(N=63 * 12, seed=3, columns=12)
    fv = FlyVis(m, B=2)
    lum = np.linspace(0, 1, 12).astype(np.float32)
    fv.setInput(lum, 1)
    x1 = fv.read("x", 1)
    for ix in m["inputIdx"].values():
        np.testing.assert_array_equal(x1[ix], lum[:ix.shape[0]])
    assert not fv.read("x", 0).any()
    fv.set_input([3, 4, 3], [1.0, 2.0, 5.0], 0)
    x0 = fv.read("x", 0)
    assert x0[3] == 5.0 and x0[4] == 2.0
    fv.step(5)
    assert not np.array_equal(fv.v(1), m["bias"])
    fv.reset(1)
    np.testing.assert_array_equal(fv.v(1), m["bias"])
    assert not np.array_equal(fv.v(0), m["bias"])
    from flybrain import _native as nat
    with pytest.raises(nat.FlyBrainError):
        fv.set_input([m["N"]], [1.0], 0)
