"""The batched ensemble at full scale (N=165,122): trials built exactly as the benchmark builds
them (flybrain.ensemble: own seed, type gains compiled into the weights on the device, drive set,
uneven length) run in one uneven launch; the shortest, the median and the longest trial are
compared bit for bit with oracle runs of the same trial (the compiled weights read back from the
device, the oracle brains advanced in parallel over the host cores). Tolerance: none."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("v", "gE", "gI", "refr", "trace", "adapt", "res", "spikeCount")


@pytest.mark.slow
def test_full_scale_ensemble_trials_match_the_oracle():
    from oracle import oracle as O
    from flybrain import SYNTH_PARAMS, workload
    from flybrain.ensemble import build_ensemble, ensemble_spec

    g, _, _, _ = workload("full", seed=1)
    p = dict(SYNTH_PARAMS, wSyn=0.275, inhGain=1.0, minSyn=1)
    spec = ensemble_spec(g.N, 16, seed=7)
    batch, graphs, trials = build_ensemble(g, spec, p)
    steps = spec["steps"]
    batch.step_uneven(steps)
    order = np.argsort(steps, kind="stable")
    picks = [int(order[0]), int(order[len(order) // 2]), int(order[-1])]
    brains = []
    for b in picks:
        w, s = graphs[b].read()
        ob = O.OracleBrain(g.N, g.indptr, g.indices, w, s, p, seed=int(spec["seeds"][b]))
        idx, hz = spec["drives"][b]
        for i, h in zip(idx.tolist(), hz.tolist()):
            ob.setDriveOne(i, h)
        brains.append(ob)
    O.run_many(brains, steps[picks])
    for ob, b in zip(brains, picks):
        for f in FIELDS:
            assert getattr(ob, f).tobytes() == batch.read(f, b).tobytes(), (b, int(steps[b]), f)
        h = ob._pull()
        np.testing.assert_array_equal(batch.fired(b), ob.ring[h.lastSlot * g.N: h.lastSlot * g.N + h.nFired])
        sc = batch.scalars(b)
        assert (sc["rng"], sc["head"]) == (h.rng, h.head), b
        assert int(ob.spikeCount.sum()) > 0
