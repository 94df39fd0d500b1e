"""The delay-scheduled step kernel (FB_SCHEDULE_LAGGED, fly-brain_gb300/csrc/fb_lagged.cu)
against the reference's golden outputs and the oracle: rasters and state bit for bit, across
launch boundaries (spikes in flight handed over through the ring), mixed with the grid kernel,
with background events, depression and host injections between launches."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from scenarios import final_state, load_case, oracle_runner, run_scenario
from test_step_gpu import assert_same, gpu_stepwise, make_gpu_brain

pytestmark = pytest.mark.gpu
CASES = sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz") and not f.startswith("presynaptic"))


def lagged_chunks(chunk=64):
    """n steps as launches of at most `chunk` steps on the lagged kernel, each logged."""
    from flybrain import _native as nat

    def run(brain, n):
        b = brain._batch
        b.set_schedule(nat.FB_SCHEDULE_LAGGED)
        counts, raster = [], []
        left = n
        while left > 0:
            c = min(chunk, left)
            b.record(c, 1 << 22)
            brain.run(c)
            assert b.last_schedule() == nat.FB_SCHEDULE_LAGGED
            k, r = b.spike_log(0, c, 1 << 22)
            b.record(0, 0)
            counts.append(k)
            raster.append(r)
            left -= c
        if not counts:
            return np.zeros(0, np.int32), np.zeros(0, np.int32)
        return np.concatenate(counts), np.concatenate(raster)
    return run


@pytest.mark.parametrize("case", CASES)
def test_golden_lagged(case):
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, case))
    brain = make_gpu_brain(meta, g)
    got = run_scenario(brain, meta["script"], lagged_chunks(64))
    assert_same(blocks, got, state, final_state(brain))


@pytest.mark.parametrize("case", ["cuba_synth.npz", "background_inject.npz"])
def test_golden_lagged_odd_launches(case):
    """Launch lengths that do not divide the delay: 7 steps (shorter than the delay) and 41."""
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, case))
    for chunk in (7, 41):
        brain = make_gpu_brain(meta, g)
        got = run_scenario(brain, meta["script"], lagged_chunks(chunk))
        assert_same(blocks, got, state, final_state(brain))


def test_golden_mixed_schedules():
    """Lagged launches, single grid-kernel steps and longer grid launches interleaved."""
    from flybrain import _native as nat
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, "coba_defaults.npz"))
    brain = make_gpu_brain(meta, g)
    lag = lagged_chunks(50)

    def mixed(br, n):
        counts, raster, left, k = [], [], n, 0
        while left > 0:
            b = br._batch
            if k % 3 == 0:
                c = min(50, left)
                cc, rr = lag(br, c)
            elif k % 3 == 1:
                c = min(3, left)
                b.set_schedule(nat.FB_SCHEDULE_GRID)
                cc, rr = gpu_stepwise(br, c)
                assert b.last_schedule() == nat.FB_SCHEDULE_GRID
            else:
                c = min(30, left)
                b.set_schedule(nat.FB_SCHEDULE_GRID)
                b.record(c, 1 << 22)
                br.run(c)
                cc, rr = b.spike_log(0, c, 1 << 22)
                b.record(0, 0)
            counts.append(cc)
            raster.append(rr)
            left -= c
            k += 1
        return np.concatenate(counts), np.concatenate(raster)

    got = run_scenario(brain, meta["script"], mixed)
    assert_same(blocks, got, state, final_state(brain))


def test_small_workload_long_launches():
    """N=20,000, 150 Hz into 1%: 4,000 steps as four 1,000-step launches (AUTO picks the lagged
    kernel); after each launch the state, spike counts and the fired lists still in flight (the
    ring) equal the oracle's."""
    from oracle import oracle as O
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda, workload
    from flybrain import _native as nat
    g, idx, hz, _ = workload("small")
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, SYNTH_PARAMS, seed=1)
    gb = LIFCuda(DeviceGraph(g), SYNTH_PARAMS, seed=1)
    for i, h in zip(idx.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
        gb.setDriveOne(i, h)
    for _ in range(4):
        ob.run(1000)
        gb.run(1000)
        assert gb._batch.last_schedule() == nat.FB_SCHEDULE_LAGGED
        s0, s1 = final_state(ob), final_state(gb)
        for k in s0:
            assert s0[k].tobytes() == s1[k].tobytes(), k
        h = ob._pull()
        np.testing.assert_array_equal(gb._batch.fired(0), ob.ring[h.lastSlot * g.N: h.lastSlot * g.N + h.nFired])
    # the next steps, one launch each (grid kernel), continue from the handed-over ring
    for _ in range(30):
        np.testing.assert_array_equal(gb.step(), ob.step())


def test_lagged_refuses_presynaptic_inhibition():
    from flybrain import _native as nat
    meta, g, blocks, state = load_case(os.path.join(GOLDEN, "presynaptic_inhibition.npz"))
    brain = make_gpu_brain(meta, g)
    brain._batch.set_schedule(nat.FB_SCHEDULE_LAGGED)
    with pytest.raises(nat.FlyBrainError):
        brain.run(100)
    brain._batch.set_schedule(nat.FB_SCHEDULE_AUTO)
    brain.run(100)
    assert brain._batch.last_schedule() == nat.FB_SCHEDULE_GRID
