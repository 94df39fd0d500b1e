"""The native decoders of the reference's compressed data files (fb_codec.cu): FLYG, the
connectome CSR (src/codec/graph.js), and FLYN, the per-neuron table (src/codec/neurons.js).

Pinned on the reference's own files when its data directory is present: graph.flyg decodes to
graph_w3.bin and neurons.flyn to neurons.bin, array for array, and the test encoder
(tests/flyg_encode.py) reproduces neurons.flyn byte for byte. Synthetic tables cover the edge
cases through encode -> native decode round trips. Host code only: no device is used."""
import os
import shutil

import numpy as np
import pytest

from flyg_encode import encode_flyg, encode_flyn

from refpaths import REF_DATA
HAVE_REF = os.path.exists(os.path.join(REF_DATA, "graph.flyg"))


def _decode_graph(buf: bytes):
    import ctypes as C
    from flybrain import _native as nat
    L = nat.load()
    raw = np.frombuffer(buf, np.uint8).copy()
    h = nat.FbFlygHeader()
    nat.check(L.fb_flyg_sizes(nat.ptr(raw), raw.shape[0], C.byref(h)))
    out = (np.zeros(h.N + 1, np.uint32), np.zeros(h.E, np.uint32), np.zeros(h.E, np.uint16))
    nat.check(L.fb_flyg_decode(nat.ptr(raw), raw.shape[0], *(nat.ptr(a) for a in out)))
    return out


def _csr(rows):
    indptr = np.zeros(len(rows) + 1, np.uint32)
    indptr[1:] = np.cumsum([len(r) for r in rows])
    idx = np.concatenate([np.sort(np.asarray(r, np.int64)) for r in rows]).astype(np.uint32) if indptr[-1] else \
        np.zeros(0, np.uint32)
    return indptr, idx


CASES = ["random", "empty_rows", "one_neuron", "no_edges", "dense_rows", "heavy"]


@pytest.mark.parametrize("case", CASES)
def test_flyg_round_trip(case):
    rng = np.random.default_rng(CASES.index(case))
    mw = 3
    if case == "random":
        N = 900
        rows = [rng.choice(N, int(rng.integers(0, 40)), replace=False) for _ in range(N)]
    elif case == "empty_rows":
        N = 300
        rows = [rng.choice(N, 5, replace=False) if i % 7 == 0 else [] for i in range(N)]
    elif case == "one_neuron":
        N, rows = 1, [[0]]
    elif case == "no_edges":
        N, rows = 50, [[] for _ in range(50)]
    elif case == "dense_rows":  # neighbouring rows share most targets (the copy bits)
        N = 200
        base = rng.choice(N, 120, replace=False)
        rows = [np.unique(np.concatenate([base[rng.random(120) < 0.9], rng.choice(N, 5)])) for _ in range(N)]
    else:  # synapse counts up to the u16 maximum
        N = 120
        rows = [rng.choice(N, 30, replace=False) for _ in range(N)]
    indptr, idx = _csr(rows)
    E = int(indptr[-1])
    w = rng.integers(mw, 70, E).astype(np.uint16)
    if case == "heavy" and E:
        w[::5] = 65535
    for order in (None, rng.permutation(N)):
        dec = _decode_graph(encode_flyg(N, indptr, idx, w, mw, order))
        np.testing.assert_array_equal(dec[0], indptr)
        np.testing.assert_array_equal(dec[1], idx)
        np.testing.assert_array_equal(dec[2], w)


def test_flyn_round_trip(tmp_path):
    from flybrain.connectome import load_flyn
    rng = np.random.default_rng(4)
    N = 2000
    ids = np.cumsum(rng.integers(1, 10 ** 6, N)).astype(np.int64) + 10 ** 9
    soma = rng.integers(-5000, 90000, (N, 3)).astype(np.float32)
    soma[rng.random(N) < 0.3] = np.nan
    cls = rng.integers(0, 900, N).astype(np.uint16)
    nt = rng.integers(0, 8, N).astype(np.uint8)
    sc = rng.integers(0, 27, N).astype(np.uint8)
    side = rng.integers(0, 3, N).astype(np.uint8)
    p = str(tmp_path / "roundtrip.flyn")
    with open(p, "wb") as f:
        f.write(encode_flyn(ids, soma, cls, nt, sc, side))
    t = load_flyn(p)
    np.testing.assert_array_equal(t["bodyIds"], ids)
    np.testing.assert_array_equal(t["soma"], soma)
    for k, v in (("cls", cls), ("nt", nt), ("sc", sc), ("side", side)):
        np.testing.assert_array_equal(t[k], v)


def test_bad_streams_are_rejected():
    from flybrain import _native as nat
    indptr, idx = _csr([[1, 2], [0], []])
    good = encode_flyg(3, indptr, idx, np.array([3, 4, 5], np.uint16), 3)
    with pytest.raises(nat.FlyBrainError, match="FLYG"):
        _decode_graph(b"XXXX" + good[4:])
    with pytest.raises(nat.FlyBrainError, match="header"):
        _decode_graph(good[:12])
    big = np.frombuffer(good, np.uint8).copy()
    big[8:12] = np.frombuffer(np.uint32(1 << 19).tobytes(), np.uint8)  # N beyond the 18-bit field
    with pytest.raises(nat.FlyBrainError, match="18-bit"):
        _decode_graph(big.tobytes())
    # a damaged body is either rejected or decodes to some graph; it never reads or writes out of bounds
    rng = np.random.default_rng(0)
    for _ in range(20):
        bad = np.frombuffer(good, np.uint8).copy()
        bad[20 + int(rng.integers(0, len(good) - 20))] ^= np.uint8(1 << int(rng.integers(0, 8)))
        try:
            _decode_graph(bad.tobytes())
        except nat.FlyBrainError:
            pass


@pytest.mark.skipif(not HAVE_REF, reason="no connectome data directory")
def test_reference_graph_flyg_is_graph_w3():
    from flybrain.connectome import load_flyg, load_graph
    f = load_flyg(os.path.join(REF_DATA, "graph.flyg"))
    g = load_graph(os.path.join(REF_DATA, f"graph_w{f['min_weight']}.bin"))
    assert (f["N"], f["E"]) == (g["N"], g["E"]) == (165122, 10511038)
    for k in ("indptr", "indices", "counts"):
        np.testing.assert_array_equal(f[k], g[k])


@pytest.mark.skipif(not HAVE_REF, reason="no connectome data directory")
def test_reference_neurons_flyn_is_neurons_bin():
    from flybrain.connectome import load_flyn, load_neurons
    t = load_flyn(os.path.join(REF_DATA, "neurons.flyn"))
    b = load_neurons(os.path.join(REF_DATA, "neurons.bin"), t["N"])
    for k in ("bodyIds", "cls", "nt", "sc", "side"):
        np.testing.assert_array_equal(t[k], b[k])
    np.testing.assert_array_equal(t["soma"], b["soma"])
    # the test encoder writes the reference's file byte for byte
    with open(os.path.join(REF_DATA, "neurons.flyn"), "rb") as f:
        assert encode_flyn(b["bodyIds"], b["soma"], b["cls"], b["nt"], b["sc"], b["side"]) == f.read()


@pytest.mark.skipif(not HAVE_REF, reason="no connectome data directory")
def test_data_directory_with_compressed_files_only(tmp_path):
    """A deployed data directory holds graph.flyg and neurons.flyn without the flat tables: the
    loader reads those and derives the degrees."""
    from flybrain.connectome import load_connectome
    for fn in ("meta.json", "graph.flyg", "neurons.flyn", "neuron_size.bin", "ntsign.bin"):
        shutil.copy(os.path.join(REF_DATA, fn), tmp_path / fn)
    c = load_connectome(str(tmp_path))
    ref = load_connectome(REF_DATA)
    for k in ("indptr", "indices", "counts", "bodyIds", "cls", "nt", "sc", "side", "indeg", "outdeg"):
        np.testing.assert_array_equal(c[k], ref[k])
    np.testing.assert_array_equal(c["soma"], ref["soma"])


def test_loader_reads_compressed_tables_without_the_flat_ones(tmp_path):
    """A synthetic data directory written both ways: the loader's result from graph.flyg and
    neurons.flyn alone equals its result from the flat tables."""
    from flybrain.connectome import load_connectome, load_neurons, write_connectome
    from flybrain.synth import synth_graph
    g = synth_graph(1500, 8)
    nt = np.random.default_rng(8).integers(0, 8, g.N).astype(np.uint8)
    flat, comp = tmp_path / "flat", tmp_path / "comp"
    write_connectome(str(flat), g.N, g.indptr, g.indices, g.counts, nt, min_weight=3)
    ref = load_connectome(str(flat))
    comp.mkdir()
    shutil.copy(flat / "meta.json", comp / "meta.json")
    w = np.minimum(g.counts, 65535).astype(np.uint16)
    (comp / "graph.flyg").write_bytes(encode_flyg(g.N, g.indptr, g.indices, w, 3,
                                                  np.random.default_rng(1).permutation(g.N)))
    t = load_neurons(str(flat / "neurons.bin"), g.N)
    t["soma"][::7] = np.nan
    (comp / "neurons.flyn").write_bytes(encode_flyn(t["bodyIds"], t["soma"], t["cls"], t["nt"], t["sc"], t["side"]))
    c = load_connectome(str(comp))
    for k in ("N", "E", "min_weight"):
        assert c[k] == ref[k], k
    for k in ("indptr", "indices", "counts", "bodyIds", "cls", "nt", "sc", "side", "indeg", "outdeg"):
        np.testing.assert_array_equal(c[k], ref[k])
    np.testing.assert_array_equal(c["soma"], t["soma"])
    assert c["size"] is None and c["ntsign"] is None
