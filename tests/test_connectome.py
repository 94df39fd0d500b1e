"""The connectome table reader (flybrain/connectome.py) on the reference's own data directory
(when present) and on tables written in the same layouts."""
import os

import numpy as np
import pytest

from refpaths import REF_DATA


def test_round_trip(tmp_path):
    from flybrain.connectome import load_connectome, write_connectome
    from flybrain.synth import synth_graph
    g = synth_graph(700, 3)
    nt = np.random.default_rng(3).integers(0, 8, g.N).astype(np.uint8)
    write_connectome(str(tmp_path), g.N, g.indptr, g.indices, g.counts, nt)
    c = load_connectome(str(tmp_path))
    assert (c["N"], c["E"]) == (g.N, g.E)
    np.testing.assert_array_equal(c["indptr"], g.indptr)
    np.testing.assert_array_equal(c["indices"], g.indices)
    np.testing.assert_array_equal(c["counts"], g.counts)
    np.testing.assert_array_equal(c["nt"], nt)
    np.testing.assert_array_equal(c["outdeg"], np.diff(g.indptr.astype(np.int64)))
    assert c["size"] is None and c["ntsign"] is None


def test_truncated_and_inconsistent_tables_are_rejected(tmp_path):
    from flybrain.connectome import load_connectome, load_graph, write_connectome
    from flybrain.synth import synth_graph
    g = synth_graph(300, 4)
    write_connectome(str(tmp_path), g.N, g.indptr, g.indices, g.counts, np.zeros(g.N, np.uint8))
    p = os.path.join(str(tmp_path), "graph_w3.bin")
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-10])
    with pytest.raises(ValueError, match="too short"):
        load_graph(p)
    bad = bytearray(raw)
    bad[8 + 4 * g.N: 8 + 4 * (g.N + 1)] = np.uint32(5).tobytes()  # indptr[N] != E
    open(p, "wb").write(bytes(bad))
    with pytest.raises(ValueError, match="CSR"):
        load_connectome(str(tmp_path))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DATA, "graph_w3.bin")), reason="reference data absent")
def test_reference_tables():
    """The reference's whole-CNS tables: 165,122 neurons, the metadata's edge count, counts at or
    above the file's minimum weight, per-neuron degrees consistent with the graph."""
    from flybrain.connectome import load_connectome, pre_sign
    c = load_connectome(REF_DATA)
    assert c["N"] == 165122 and c["E"] == c["meta"]["edges"]
    assert int(c["counts"].min()) >= c["min_weight"]
    np.testing.assert_array_equal(c["outdeg"], np.diff(c["indptr"].astype(np.int64)))
    np.testing.assert_array_equal(c["indeg"], np.bincount(c["indices"], minlength=c["N"]))
    assert c["size"] is not None and c["size"].shape == (c["N"],)
    s = pre_sign(c)
    assert set(np.unique(s).tolist()) <= {-1.0, 0.0, 1.0}
    # rows sorted by target (scripts/prep_graph.py:40)
    r = c["indices"][c["indptr"][1000]: c["indptr"][1001]]
    assert np.all(np.diff(r.astype(np.int64)) > 0)
