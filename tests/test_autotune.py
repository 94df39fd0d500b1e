"""The autotuner's search and cache on the host, with a fake batch whose step time depends on the
launch shape (no GPU)."""
import pytest


class FakeBrains:
    B = 4

    def __init__(self):
        self.shape = (2, 1)
        self.sched = []

    def tuning(self):
        return dict(blocks_per_sm=self.shape[0], item_chunks=self.shape[1], max_blocks_per_sm=3, sms=152)

    def set_tuning(self, b=0, c=0):
        self.shape = (b or self.shape[0], c or self.shape[1])

    def set_schedule(self, s):
        self.sched.append(s)

    def step(self, n):
        self.n = n

    def last_ms(self):
        b, c = self.shape
        return self.n * (1.0 + abs(b - 2) * 0.3 + abs(c - 4) * 0.1)


def test_tune_brains_picks_the_fastest_and_caches(tmp_path, monkeypatch):
    from flybrain import _native as nat
    from flybrain import autotune
    monkeypatch.setenv("FLYBRAIN_TUNE_CACHE", str(tmp_path / "t.json"))
    monkeypatch.setattr(autotune, "_device", lambda: "fake")
    fb = FakeBrains()
    r = autotune.tune_brains(fb, steps=10, item_chunks=(1, 2, 4, 8))
    assert (r["blocks_per_sm"], r["item_chunks"]) == (2, 4) and fb.shape == (2, 4)
    assert len(r["table"]) == 12 and not r["cached"]
    assert fb.sched == [nat.FB_SCHEDULE_GRID, nat.FB_SCHEDULE_AUTO]
    fb2 = FakeBrains()
    r2 = autotune.tune_brains(fb2, steps=10)
    assert r2["cached"] and fb2.shape == (2, 4)


class FakeDiff:
    B = 2
    N = [100, 100]

    def __init__(self, clock):
        self.p = dict(checkpoint=100)
        self.tune = (0, 0)
        self.clock = clock
        self.K = 100

    def set_tuning(self, nb=0, ab=0, step_launches=None):
        self.tune = (nb, ab)
        self.tuning = dict(neuron_blocks=nb, arrival_blocks=ab, step_launches=step_launches)

    def forward(self, steps, seeds, record=True, counts=False, checkpoint=100):
        self.K = checkpoint

    def backward(self, dLs, readouts=None, edge=True):
        assert self.tuning["step_launches"] is True  # candidates are timed with step launches
        nb, ab = self.tune
        self.clock[0] += 1.0 + abs(self.K - 50) / 100 + (0.2 if nb != 1 else 0) + (0.1 if ab != 8 else 0)


def test_tune_diff_coordinate_descent(tmp_path, monkeypatch):
    from flybrain import autotune
    monkeypatch.setenv("FLYBRAIN_TUNE_CACHE", str(tmp_path / "t.json"))
    monkeypatch.setattr(autotune, "_device", lambda: "fake")
    clock = [0.0]
    monkeypatch.setattr(autotune, "_sync", lambda: None)
    monkeypatch.setattr(autotune.time, "perf_counter", lambda: clock[0])
    fd = FakeDiff(clock)
    r = autotune.tune_diff(fd, [10, 10], [1, 2], [None, None], Ks=(25, 50, 200), neuron_blocks=(1, 4),
                           arrival_blocks=(2, 8))
    assert (r["checkpoint"], r["neuron_blocks"], r["arrival_blocks"]) == (50, 1, 8)
    assert fd.p["checkpoint"] == 50 and fd.tune == (1, 8)
    assert fd.tuning["step_launches"] is False  # the launch mode is restored
    assert autotune.tune_diff(FakeDiff(clock), [10, 10], [1, 2], [None, None])["cached"]


def test_unwritable_cache_is_not_an_error(tmp_path, monkeypatch):
    from flybrain import autotune
    bad = tmp_path / "file"
    bad.write_text("x")
    monkeypatch.setenv("FLYBRAIN_TUNE_CACHE", str(bad / "sub" / "t.json"))
    monkeypatch.setattr(autotune, "_device", lambda: "fake")
    r = autotune.tune_brains(FakeBrains(), steps=5, item_chunks=(4,))
    assert r["item_chunks"] == 4
