"""The neuromodulation controller (flybrain/neuromod.py, after src/sim/neuromod.js) on a recording
brain: the modulatory cells and octopamine targets it finds, the conductances it adds each
millisecond, the rate filter and thresholds every 10 ms, the threshold (or gain) field every
50 ms, and the operators and blocks. Values are checked against the reference's formulas worked
out here in double precision with float32 stores. No JavaScript engine is available, so the
controller is not pinned on the reference's own output."""
import math

import numpy as np
import pytest

TYPES = ["OA-VUMa1", "OA-AL2i1", "IPC", "KCab", "T4a", "OA-X", "L1", "MN9"]


def _data():
    # rows by presynaptic neuron: (target, synapse count)
    rows = {0: [(3, 9), (4, 3), (6, 12)], 1: [(4, 7), (5, 6)], 2: [(0, 8)], 5: [(3, 5), (7, 20)], 6: [(1, 4)]}
    N = len(TYPES)
    indptr = np.zeros(N + 1, np.uint32)
    idx, cnt = [], []
    for i in range(N):
        for q, c in rows.get(i, []):
            idx.append(q)
            cnt.append(c)
        indptr[i + 1] = len(idx)
    return dict(N=N, indptr=indptr, indices=np.array(idx, np.uint32), counts=np.array(cnt, np.uint16),
                sc=np.array([0, 1, 0, 0, 1, 0, 1, 2], np.uint8),
                meta=dict(types=TYPES, superclasses=["central", "ol_intrinsic", "descending"]))


class Brain:
    """Records the LIFWasm calls; setThr stores float32, addG accumulates in float32."""

    def __init__(self, N):
        self.thr = np.zeros(N, np.float32)
        self.thr[3] = 7.319  # a Kenyon cell's class threshold
        self.spikeCount = np.zeros(N, np.uint32)
        self.sign = np.array([1, -1, 1, 1, -1, 1, 1, -1], np.float32) * np.float32(0.3)
        self.gE = np.zeros(N, np.float32)
        self.gI = np.zeros(N, np.float32)
        self.calls = []

    def setThr(self, i, mv):
        self.thr[i] = mv

    def addG(self, i, e, ii=0.0):
        self.calls.append((i, e, ii))
        self.gE[i] = np.float32(float(self.gE[i]) + e)
        self.gI[i] = np.float32(float(self.gI[i]) + (ii or 0.0))


def sig(x, h, w):
    return 1 / (1 + math.exp(-(x - h) / w))


def test_cells_targets_and_resting_thresholds():
    from flybrain.neuromod import Neuromod
    b = Brain(8)
    nm = Neuromod(_data(), b, calib=dict(oaThr={"0": 25.268, "5": 7.301}, ipcThr={"2": 11.5}), min_syn=5)
    np.testing.assert_array_equal(nm.cells, [0, 1, 5, 2])  # OA neurons in index order, then IPCs
    assert nm.nOA == 3 and nm.akhr.tolist() == [0] and nm.optic.tolist() == [1] and nm.ipc.tolist() == [2]
    # targets in order of first appearance over the OA rows, edges below minSyn dropped
    np.testing.assert_array_equal(nm.targets, [3, 6, 4, 5, 7])
    assert [r.tolist() for r in nm.rows] == [[0, 9, 1, 12], [2, 7, 3, 6], [0, 5, 4, 20]]
    np.testing.assert_array_equal(nm.is_cell, [0, 0, 0, 1, 0])
    np.testing.assert_array_equal(nm.cell_target, [-1, -1, 3, -1])
    np.testing.assert_array_equal(nm.thr0, np.float32([7.319, 0, 0, 0, 0]))
    # resting thresholds with the slow AHP at the fed rates: base + sfa * r
    f = np.float32
    assert b.thr[0] == f(float(f(25.268)) + 0.5 * 2) and b.thr[1] == f(0 + 0.5 * 2)
    assert b.thr[5] == f(float(f(7.301)) + 0.5 * 2) and b.thr[2] == f(float(f(11.5)) + 0.5 * 5)


def test_millisecond_drive_and_rate_filter():
    from flybrain.neuromod import Neuromod
    b = Brain(8)
    nm = Neuromod(_data(), b)
    sugar, loco = 0.3, 0.5
    nm.update(1, sugar, loco)
    akh = (sig(-sugar, -0.4, 0.15) - 0) * 1 / 5000
    want = [(2, 4 * sig(sugar, 0.4, 0.15) * 1, 0.0), (0, 3 * akh * 1, -(1 * 1.0 * 1)), (1, 6 * loco * 1, 0.0)]
    assert len(b.calls) == 3
    for (i, e, ii), (wi, we, wii) in zip(b.calls, want):
        assert i == wi and e == we and ii == wii
    assert nm.akh == akh
    # 10 ms in: the rate filter with these spike counts
    b.spikeCount[[0, 1, 5, 2]] = [3, 0, 1, 2]
    for _ in range(9):
        nm.update(1, sugar)
    f = np.float32
    k = 10 / 2000
    r0 = [f(2 + ((3 - 0) * 1000 / 10 - 2) * k), f(2 + (0 - 2) * k), f(2 + ((1 - 0) * 1000 / 10 - 2) * k),
          f(5 + ((2 - 0) * 1000 / 10 - 5) * k)]
    np.testing.assert_array_equal(nm.r, np.array(r0, np.float32))
    dilp = 1 + (min(1.5, float(r0[3]) / 1 / 5) - 1) * 10 / 10000
    assert nm.dilp == dilp
    np.testing.assert_array_equal(b.thr[[0, 1, 5, 2]], np.array([f(0 + 0.5 * float(r)) for r in r0], np.float32))


def test_threshold_field_every_50_ms():
    from flybrain.neuromod import Neuromod
    b = Brain(8)
    nm = Neuromod(_data(), b)
    for _ in range(50):
        nm.update(1, 0.85)
    f = np.float32
    c = nm.c.copy()  # OA release after five filter updates
    x = np.zeros(5, np.float32)
    for n, row in enumerate(nm.rows):
        for m in range(0, len(row), 2):
            x[row[m]] = f(float(x[row[m]]) + int(row[m + 1]) * float(c[n]))
    shift = np.array([f(2 * float(v) / (float(v) + 400)) for v in x], np.float32)
    np.testing.assert_array_equal(nm.x, x)
    np.testing.assert_array_equal(nm.shift, shift)
    # non-cell targets: resting threshold minus the shift (the Kenyon cell keeps its class offset)
    for m, q in enumerate(nm.targets.tolist()):
        if not nm.is_cell[m]:
            assert b.thr[q] == f(float(nm.thr0[m]) - float(shift[m])), q
    assert b.thr[3] < np.float32(7.319)
    # the OA cell that is itself a target (5) gets the shift through its own threshold at the next release
    for _ in range(10):
        nm.update(1, 0.85)
    n5 = 2
    assert b.thr[5] == f(float(nm.base[n5]) + 0.5 * float(nm.r[n5]) - float(nm.shift[3]))


def test_operators_and_blocks():
    from flybrain.neuromod import Neuromod
    # synFast: no field on the targets
    b = Brain(8)
    nm = Neuromod(_data(), b, params=dict(oaMode="synFast"))
    for _ in range(50):
        nm.update(1, 0.5)
    assert (nm.shift == 0).all() and b.thr[4] == 0 and b.thr[3] == np.float32(7.319)
    # block 'OA': the field is never computed
    b = Brain(8)
    nm = Neuromod(_data(), b, block="OA")
    for _ in range(100):
        nm.update(1, 0.5)
    assert (nm.x == 0).all() and nm.arousal == 0.0
    # blocks 'AKHR' / 'InR': no AKH / no insulin conductance onto the AKHR cells
    for blk, which in (("AKHR", 1), ("InR", 2)):
        b = Brain(8)
        nm = Neuromod(_data(), b, block=blk)
        nm.update(1, 0.1)
        call = [c for c in b.calls if c[0] == 0][0]
        assert call[which] == 0 or call[which] == -0.0
    # thrTyped: only the listed types feel the field
    b = Brain(8)
    nm = Neuromod(_data(), b, params=dict(oaMode="thrTyped", oaTargets=dict(thrTyped=["T4a", "L.*"])))
    for _ in range(50):
        nm.update(1, 0.2)
    np.testing.assert_array_equal(nm.field_mask, [0, 1, 1, 0, 0])
    assert nm.shift[0] == 0 and nm.shift[1] > 0 and b.thr[7] == 0
    # gainField: outgoing gain of the typed sets through the graph sign, thresholds untouched
    b = Brain(8)
    s0 = b.sign.copy()
    nm = Neuromod(_data(), b, params=dict(oaMode="gainField",
                                          oaTargets=dict(gainField=dict(superclasses=["ol_intrinsic"], types=["MN9"]))))
    for _ in range(50):
        nm.update(1, 0.2)
    np.testing.assert_array_equal(nm.field_mask, [0, 1, 1, 0, 1])
    f = np.float32
    for m, q in enumerate(nm.targets.tolist()):
        xm = float(nm.x[m])
        want = f(float(s0[q]) * (1 + 2 * xm / (xm + 400))) if nm.field_mask[m] else s0[q]
        assert b.sign[q] == want, q
    assert b.thr[4] == 0 and (nm.shift == 0).all()
    nm.reset()
    np.testing.assert_array_equal(b.sign, s0)
    with pytest.raises(ValueError):
        Neuromod(_data(), Brain(8), params=dict(oaMode="gainField"))
