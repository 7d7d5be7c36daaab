"""The batch autotuner's host logic on the CPU (natrix_gb300/core/batch.py):
per size class it times every (tile configuration, sweeps per launch)
candidate, keeps and applies the fastest, records the choice under the key of
GPU model and class signature, and a batch with the same key takes the cached
choice without timing anything.  The timing itself (CUDA events around whole
batch steps) is replaced by a cost table."""
from __future__ import annotations

import json

import pytest

from natrix_gb300.core import batch as nb


class FakeBatch(nb.FluidBatch):
    """A FluidBatch without device state: tuning is recorded, a step's time
    comes from `cost(size_class, config, sweeps_per_launch)`."""

    def __init__(self, widths, heights, cost, key="GB300|classes=[2, 0, 1]"):
        self.widths, self.heights = list(widths), list(heights)
        self.tuning = {}
        self.timed = 0
        self._cost = cost
        self._key = key
        self._handle = None

    def set_tuning(self, size_cls, config, sweeps_per_launch):
        self.tuning[int(size_cls)] = (int(config), int(sweeps_per_launch))

    def _time_steps(self, steps, dt):
        self.timed += 1
        return sum(self._cost(c, *t) for c, t in self.tuning.items())

    def sync(self):
        pass

    def _cache_key(self):
        return self._key

    def destroy(self):
        pass


BEST = {0: (1, 4), 2: (2, 8)}


def cost(cls, cfg, spl):
    # the best candidate per class is cheapest; the others cost by distance
    b = BEST[cls]
    return 1.0 + abs(cfg - b[0]) + abs(spl - b[1]) / 4.0


def test_size_classes():
    assert [nb.size_class(w, w) for w in (16, 128, 129, 256, 257, 2048)] == [0, 0, 1, 1, 2, 2]
    assert nb.size_class(64, 300) == 2  # the longer side decides


def test_autotune_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setattr(nb, "CACHE", tmp_path / "autotune.json")
    fb = FakeBatch([64, 100, 300], [64, 128, 300], cost)
    assert fb.classes() == [0, 2]
    got = fb.autotune(steps=3)
    assert got == BEST and fb.tuning == BEST
    assert fb.timed == 2 * len(nb.CANDIDATES)
    data = json.loads((tmp_path / "autotune.json").read_text())
    assert data[fb._cache_key()] == {"0": [1, 4], "2": [2, 8]}

    # same key: the cached choice is applied, nothing is timed
    other = FakeBatch([64, 100, 300], [64, 128, 300], lambda *a: pytest.fail("timed"))
    assert other.autotune() == BEST and other.timed == 0

    # another key is tuned afresh and added beside the first
    third = FakeBatch([200], [200], lambda c, cfg, spl: 1.0 + cfg + spl, key="GB300|other")
    assert third.autotune() == {1: (0, 4)}
    data = json.loads((tmp_path / "autotune.json").read_text())
    assert set(data) == {fb._cache_key(), "GB300|other"}


def test_autotune_without_cache(tmp_path, monkeypatch):
    monkeypatch.setattr(nb, "CACHE", tmp_path / "autotune.json")
    fb = FakeBatch([300, 400], [300, 100], cost)
    assert fb.autotune(cache=False) == {2: (2, 8)}
    assert not (tmp_path / "autotune.json").exists()


def test_time_steps_brackets_the_timed_steps(monkeypatch):
    """The timing itself: two untimed steps, then `steps` steps between two
    CUDA events (a fake event class that reads a step counter here)."""

    class Counting(nb.FluidBatch):
        def __init__(self):
            self.done = []
            self._handle = None

        def step(self, dt):
            self.done.append(dt)

        def destroy(self):
            pass

    fb = Counting()

    class FakeEvent:
        def __init__(self, enable_timing=False):
            assert enable_timing
            self.at = None

        def record(self):
            self.at = len(fb.done)

        def synchronize(self):
            pass

        def elapsed_time(self, end):
            return 0.5 * (end.at - self.at)  # 0.5 ms per step

    monkeypatch.setattr(nb.torch.cuda, "Event", FakeEvent)
    assert fb._time_steps(4, 0.01) == pytest.approx(0.5)
    assert fb.done == [0.01] * 6
