"""Tables in the reference's data layout, read and compiled on the device (writeGraph), then
stepped: rasters identical to the oracle's on the same tables."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tables_compile_and_run_like_the_oracle(tmp_path):
    from oracle import oracle as O
    from flybrain import LIFCuda
    from flybrain.connectome import load_connectome, pre_sign, to_device_graph, write_connectome
    from flybrain.synth import synth_graph
    g = synth_graph(3000, 21)
    rng = np.random.default_rng(21)
    nt = rng.choice([1, 2, 3, 4], g.N).astype(np.uint8)
    write_connectome(str(tmp_path), g.N, g.indptr, g.indices, g.counts, nt)
    c = load_connectome(str(tmp_path))
    p = dict(O.DEFAULTS, coba=True, wSyn=0.3, minSyn=5, dt=0.1)
    in_scale = rng.uniform(0.5, 1.0, g.N).astype(np.float32)
    sensory = (rng.random(g.N) < 0.05).astype(np.uint8)
    dg = to_device_graph(c, p, in_scale=in_scale, sensory_mask=sensory)
    W, sign = O.write_graph_f64(g.N, c["indptr"], c["indices"], c["counts"], pre_sign(c).astype(np.float64), p,
                                in_scale=in_scale, sensory_mask=sensory)
    w_dev, s_dev = dg.read()
    assert w_dev.tobytes() == np.asarray(W, np.float32).tobytes() and s_dev.tobytes() == np.asarray(sign, np.float32).tobytes()
    brain = LIFCuda(dg, p, seed=4)
    ob = O.OracleBrain(g.N, c["indptr"], c["indices"], W, sign, p, seed=4)
    drv = rng.choice(g.N, 80, replace=False)
    for i in drv:
        brain.setDriveOne(int(i), 200.0)
        ob.setDriveOne(int(i), 200.0)
    brain._batch.record(600, 1 << 20)
    brain.run(600)
    c1, r1 = brain._batch.spike_log(0, 600, 1 << 20)
    c0, r0 = ob.run(600, raster=True)
    np.testing.assert_array_equal(c1, c0)
    np.testing.assert_array_equal(r1, r0)
