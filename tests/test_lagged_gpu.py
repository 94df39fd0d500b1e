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


def assert_same_as_oracle(gb, ob, where=""):
    """Every state word, spike count, the generator state, the ring head and every fired list
    still in flight of the GPU brain equal the oracle brain's."""
    s0, s1 = final_state(ob), final_state(gb)
    for k in s0:
        assert s0[k].tobytes() == s1[k].tobytes(), (where, k)
    h = ob._pull()
    sc = gb._batch.scalars(0)
    assert (sc["rng"], sc["head"], sc["nFired"], sc["lastSlot"]) == (h.rng, h.head, h.nFired, h.lastSlot), where
    lists, counts, head = gb._batch.ring(0)
    assert head == h.head, where
    np.testing.assert_array_equal(counts, ob.ringCount, err_msg=str(where))
    N = ob.N
    for s in range(counts.shape[0]):
        np.testing.assert_array_equal(lists[s, :counts[s]], ob.ring[s * N: s * N + counts[s]], err_msg=f"{where} slot {s}")


def _long_launches(name, launches, length, seed=1):
    from oracle import oracle as O
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda, workload
    from flybrain import _native as nat
    g, idx, hz, _ = workload(name)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, SYNTH_PARAMS, seed=seed)
    gb = LIFCuda(DeviceGraph(g), SYNTH_PARAMS, seed=seed)
    for i, h in zip(idx.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
        gb.setDriveOne(i, h)
    gb._batch.set_schedule(nat.FB_SCHEDULE_LAGGED)
    spikes = 0
    for k in range(launches):
        ob.run(length)
        gb.run(length)
        assert gb._batch.last_schedule() == nat.FB_SCHEDULE_LAGGED
        assert_same_as_oracle(gb, ob, (name, k))
        spikes = int(ob.spikeCount.sum())
    return ob, gb, spikes


def test_small_workload_long_launches():
    """N=20,000, 150 Hz into 1%: the whole 1,000 ms window (10,000 steps) as ten 1,000-step
    launches of the delay-scheduled kernel; after each launch the state, spike counts, generator
    state and every fired list still in flight (the ring) equal the oracle's. The next steps, one
    grid-kernel launch each, continue from the handed-over ring."""
    from flybrain import _native as nat
    ob, gb, spikes = _long_launches("small", 10, 1000)
    assert spikes > 0
    gb._batch.set_schedule(nat.FB_SCHEDULE_AUTO)
    for _ in range(30):
        np.testing.assert_array_equal(gb.step(), ob.step())


@pytest.mark.slow
def test_full_scale_whole_window_long_launches():
    """The headline workload: N=165,122 (~11M edges), 2,000 drivers at 100-200 Hz, the whole
    2,000 ms window (20,000 steps) as twenty unlogged 1,000-step launches of the delay-scheduled
    kernel -- the launches the throughput figures are measured on. After every launch every state
    word, the spike counts, the generator state, the ring head and every fired list still in
    flight equal the oracle's, bit for bit, from step 0."""
    ob, gb, spikes = _long_launches("full", 20, 1000)
    assert spikes > 400_000


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


@pytest.mark.parametrize("bg", [False, True])
def test_driven_list_split_over_two_blocks(bg):
    """A driven list long enough to be split over two driven blocks (each offsets its draws by the
    other's share of live entries), N=20,000 with 1,500 drivers (and, in one case, background
    events and depression, whose hits on driven neurons the second block collects too): three
    1,000-step launches, state, generator, ring and fired lists identical to the oracle."""
    from oracle import oracle as O
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda, drive_set, synth_graph
    from flybrain import _native as nat
    g = synth_graph(20000, 5)
    idx, hz = drive_set(g.N, 1500, 77, 80.0, 220.0)
    p = dict(SYNTH_PARAMS, bgRate=15.0, bgAmp=1.5, depU=0.1) if bg else dict(SYNTH_PARAMS)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=9)
    gb = LIFCuda(DeviceGraph(g), p, seed=9)
    for i, h in zip(idx.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
        gb.setDriveOne(i, h)
    gb._batch.set_schedule(nat.FB_SCHEDULE_LAGGED)
    for k in range(3):
        ob.run(1000)
        gb.run(1000)
        assert gb._batch.last_schedule() == nat.FB_SCHEDULE_LAGGED
        assert_same_as_oracle(gb, ob, ("split", bg, k))
    c0, r0 = ob.run(64, raster=True)
    counts, raster = lagged_chunks(64)(gb, 64)
    np.testing.assert_array_equal(counts, c0)
    np.testing.assert_array_equal(raster, r0)
    assert int(ob.spikeCount.sum()) > 10000
