"""The timeout path of the device-side waits. Every wait in the step kernels is bounded (by the
handle's timeout_us and an iteration cap) and reports FB_ETIMEOUT instead of hanging; the
reference's counterpart is its fallback when the GPU path fails (src/brainsetup.js:66-75) and its
device-lost reset (src/lifgpu.js:168).

The test arms fb_debug_trip_wait so that one block of the delay-scheduled kernel waits on a flag
nothing sets. That wait runs out after a 2 ms timeout, the other blocks leave their own bounded
waits (each checks the error word), every thread of every block leaves through the kernel's one
exit, and the call returns FB_ETIMEOUT. The failed launch leaves the brain as it was before the
call (the kernel keeps the state in shared memory until the launch completes), so the same handle
then steps on bit for bit with the oracle, and the context stays usable."""
import time

import numpy as np
import pytest

from test_lagged_gpu import assert_same_as_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("trip_at", [0, 37, 199])
def test_wait_that_runs_out_reports_timeout_and_the_brain_steps_on(trip_at):
    from oracle import oracle as O
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda, synth_graph
    from flybrain import _native as nat

    g = synth_graph(3000, 13)
    rng = np.random.default_rng(13)
    idx = rng.choice(g.N, 50, replace=False)
    p = dict(SYNTH_PARAMS, depU=0.1, bgRate=10.0, bgAmp=1.5)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=4)
    gb = LIFCuda(DeviceGraph(g), p, seed=4)
    for i in idx.tolist():
        ob.setDriveOne(i, 180.0)
        gb.setDriveOne(i, 180.0)
    b = gb._batch
    b.set_schedule(nat.FB_SCHEDULE_LAGGED)
    ob.run(150)
    gb.run(150)
    assert_same_as_oracle(gb, ob, "before")

    default = b.tuning()["timeout_us"]
    assert default == 5_000_000
    b.set_tuning(timeout_us=2000)
    assert b.tuning()["timeout_us"] == 2000
    b.trip_wait(trip_at)
    t0 = time.perf_counter()
    with pytest.raises(nat.FlyBrainError) as e:
        gb.run(200)
    elapsed = time.perf_counter() - t0
    assert e.value.code == nat.FB_ETIMEOUT, str(e.value)
    assert elapsed < 2.0, elapsed  # the 2 ms bound, not the 5 s default
    assert b.last_schedule() == nat.FB_SCHEDULE_LAGGED
    b.set_tuning(timeout_us=default)

    # the abandoned launch changed nothing: the handle steps on with the oracle, on both kernels
    assert_same_as_oracle(gb, ob, "after the timeout")
    ob.run(300)
    gb.run(300)
    assert_same_as_oracle(gb, ob, "after 300 more steps")
    b.set_schedule(nat.FB_SCHEDULE_GRID)
    for _ in range(5):
        np.testing.assert_array_equal(gb.step(), ob.step())
    assert int(ob.spikeCount.sum()) > 0


def test_trip_hook_is_consumed_by_one_launch():
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda, synth_graph
    from flybrain import _native as nat

    g = synth_graph(1500, 2)
    gb = LIFCuda(DeviceGraph(g), SYNTH_PARAMS, seed=2)
    gb.setDrive(np.arange(0, 1500, 50, dtype=np.int32), 150.0)
    b = gb._batch
    b.set_schedule(nat.FB_SCHEDULE_LAGGED)
    b.set_tuning(timeout_us=1000)
    b.trip_wait(3)
    with pytest.raises(nat.FlyBrainError):
        gb.run(40)
    gb.run(40)  # disarmed after one launch
    b.trip_wait(3)
    b.trip_wait(-1)
    gb.run(40)
    with pytest.raises(nat.FlyBrainError):
        b.set_tuning(timeout_us=-5)
