"""The oracle port (oracle/lifsim.c + the restated LIFWasm glue) reproduces the reference kernel's
golden outputs bit for bit, and matches the reference build live where it is available."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O
from scenarios import final_state, load_case, oracle_runner, run_scenario

CASES = sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def run_case(path, backend):
    meta, g, blocks, state = load_case(path)
    brain = O.OracleBrain(meta["N"], g["indptr"], g["indices"], g["W"], g["sign"], meta["params"],
                          seed=meta["seed"], backend=backend)
    got = run_scenario(brain, meta["script"], oracle_runner)
    return blocks, state, got, final_state(brain)


@pytest.mark.parametrize("case", CASES)
def test_port_matches_golden(case):
    blocks, state, got, st = run_case(os.path.join(GOLDEN, case), "port")
    assert len(got) == len(blocks)
    for (c0, r0), (c1, r1) in zip(blocks, got):
        np.testing.assert_array_equal(c1, c0)
        np.testing.assert_array_equal(r1, r0)
    for k, v in state.items():
        assert v.tobytes() == st[k].tobytes(), k  # bitwise, incl. signed zeros


def test_golden_cases_present():
    names = {c[:-4] for c in CASES}
    assert {"cuba_synth", "coba_defaults", "background_inject", "presynaptic_inhibition"} <= names
    assert sum(1 for _ in CASES) >= 4


@pytest.mark.skipif(not O.have_reference_build(), reason="reference kernel not built here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_port_matches_reference_live(seed):
    """Random parameters and drives on random synthetic graphs: port == reference lif.c."""
    from flybrain.synth import synth_graph
    rng = np.random.default_rng(seed)
    N = int(rng.integers(200, 1500))
    g = synth_graph(N, seed + 100)
    p = dict(O.DEFAULTS, dt=float(rng.choice([0.1, 0.25, 0.5])), coba=bool(rng.integers(2)),
             adaptInc=float(rng.uniform(0, 2)), depU=float(rng.uniform(0, 0.3)),
             bgRate=float(rng.uniform(0, 30)), bgAmp=float(rng.uniform(0, 2)),
             preInh=float(rng.choice([0.0, 0.3])), tRef=float(rng.uniform(0.5, 3)))
    drv = rng.choice(N, int(rng.integers(5, 60)), replace=False)
    script = [["drive", drv.tolist(), rng.uniform(10, 300, drv.shape[0]).tolist()],
              ["step", 400], ["pulse", drv[:3].tolist(), 3.0], ["step", 400]]
    out = []
    for backend in ("port", "ref"):
        b = O.OracleBrain(N, g.indptr, g.indices, g.weights, g.sign, p, seed=seed, backend=backend)
        out.append((run_scenario(b, script, oracle_runner), final_state(b)))
    (b0, s0), (b1, s1) = out
    for (c0, r0), (c1, r1) in zip(b0, b1):
        np.testing.assert_array_equal(c0, c1)
        np.testing.assert_array_equal(r0, r1)
    for k in s0:
        assert s0[k].tobytes() == s1[k].tobytes(), k


def test_header_constants_and_seed():
    """_writeHeader restatement: constants rounded once from f64; seed hash with JS semantics."""
    c = O.header_constants(dict(O.DEFAULTS, dt=0.1))
    assert c.dtype == np.float32 and c.shape == (17,)
    assert c[7] == np.float32(np.exp(-0.1 / 5.0))
    assert O.seed_state(1) == 2654435761
    assert O.seed_state(0) == 1
    # JavaScript forms seed * 2654435761 in double: above 2^53 the product is rounded (here to a
    # multiple of 64) before >>> 0; exact integer arithmetic would give 2146089093
    assert O.seed_state(123456789) == 2146089088
    assert O.seed_state(1073741823) == 2714273280
    assert O.seed_state(2097151) == 2548598351  # below 2^21 the product is exact
    assert O.n_slots(dict(delay=1.8, dt=0.1)) == 19
    assert O.n_slots(dict(delay=1.8, dt=0.5)) == 5
