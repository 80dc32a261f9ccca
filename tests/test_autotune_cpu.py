"""Host logic of the tile-shape autotuner, with fake timings and fake
handles (no GPU): the fastest candidate wins and is set, the choice is
cached per workload and reused without timing, a form whose scratch the
library refuses is skipped, the batch state is restored after every timed
candidate, and an unreadable or outdated cache entry is ignored."""
import importlib
import json

import pytest
import torch

from conftest import PKG_NAME


@pytest.fixture
def tune(monkeypatch, tmp_path):
    mod = importlib.import_module(PKG_NAME + ".autotune")
    monkeypatch.setattr(mod, "CACHE", str(tmp_path / "autotune.json"))
    monkeypatch.setattr(mod, "_key", lambda kind, sig: f"fake-gpu|{kind}|{sig}")
    return mod


class FakeSolver:
    def __init__(self, fast):
        self.fast = fast
        self.shape = None
        self.calls = 0

    def set_tiles(self, k, w, _segments, packed):
        self.shape = (k, w, packed)

    def acc(self, xm, acc, G, eps2):
        self.calls += 1


def _xm():
    return torch.zeros((5000, 4))  # only its shape and zeros_like are used


def _fake_timer(mod, monkeypatch, solver_or_batch):
    def fake_time(fn, reps):
        fn()
        return 1.0 if solver_or_batch.shape == solver_or_batch.fast else 2.0 + 0.01 * sum(solver_or_batch.shape)
    monkeypatch.setattr(mod, "_time", fake_time)


def test_tune_direct_picks_caches_and_reuses(tune, monkeypatch):
    s = FakeSolver(fast=(4, 8, 1))
    _fake_timer(tune, monkeypatch, s)
    shape, times = tune.tune_direct(s, _xm())
    assert shape == (4, 8, 1) and s.shape == (4, 8, 1)
    assert len(times) == len(tune.DIRECT_SHAPES) and s.calls == len(tune.DIRECT_SHAPES)
    with open(tune.CACHE) as f:
        cache = json.load(f)
    assert cache["fake-gpu|direct|8192"]["best"] == [4, 8, 1]
    s2 = FakeSolver(fast=(2, 4, 2))
    monkeypatch.setattr(tune, "_time", lambda fn, reps: pytest.fail("cached shape was re-timed"))
    shape2, _ = tune.tune_direct(s2, _xm())
    assert shape2 == (4, 8, 1) and s2.shape == (4, 8, 1)


def test_tune_direct_ignores_bad_cache(tune, monkeypatch):
    with open(tune.CACHE, "w") as f:
        f.write("{not json")
    s = FakeSolver(fast=(2, 4, 2))
    _fake_timer(tune, monkeypatch, s)
    assert tune.tune_direct(s, _xm())[0] == (2, 4, 2)
    with open(tune.CACHE, "w") as f:  # an entry from an older two-field format
        json.dump({"fake-gpu|direct|8192": {"best": [4, 8], "ms": {}}}, f)
    s = FakeSolver(fast=(2, 8, 0))
    _fake_timer(tune, monkeypatch, s)
    assert tune.tune_direct(s, _xm())[0] == (2, 8, 0)


class FakeBatch:
    def __init__(self, fast, refuse_variant=None):
        import numpy as np
        self.fast = fast
        self.refuse = refuse_variant
        self.tiles = (2, 4)
        self.variant = 0
        self.state = 0
        self.restores = 0
        self.n_total = 1000
        self.sizes = np.array([300, 700])
        self.runs = 0

    @property
    def shape(self):
        return (*self.tiles, self.variant)

    def interactions_per_step(self):
        return int((self.sizes ** 2).sum())

    def set_tiles(self, k, w):
        self.tiles = (k, w)

    def set_variant(self, v):
        grav_err = importlib.import_module(PKG_NAME + "._lib").GravityError
        if v == self.refuse:
            raise grav_err(1, "gb_batch_set_variant", "scratch too large")
        self.variant = v

    def state_arrays(self):
        return self.state

    def restore(self, saved):
        self.state = saved
        self.restores += 1

    def run(self, dt, nsteps, graph=True):
        self.state += 1
        self.runs += 1


def test_tune_batch_skips_refused_form_and_restores_state(tune, monkeypatch):
    b = FakeBatch(fast=(2, 4, 1), refuse_variant=1)
    _fake_timer(tune, monkeypatch, b)
    shape, times = tune.tune_batch(b)
    assert shape[2] == 0 and "2,4,1" not in times
    assert len(times) == len(tune.BATCH_SHAPES) - 1
    assert b.state == 0 and b.restores == b.runs == len(times)
    assert b.shape == shape


def test_tune_batch_prefers_symmetric_when_fastest_and_caches(tune, monkeypatch):
    b = FakeBatch(fast=(2, 4, 1))
    _fake_timer(tune, monkeypatch, b)
    assert tune.tune_batch(b)[0] == (2, 4, 1) and b.shape == (2, 4, 1)
    b2 = FakeBatch(fast=(4, 8, 0))
    monkeypatch.setattr(tune, "_time", lambda fn, reps: pytest.fail("cached shape was re-timed"))
    assert tune.tune_batch(b2)[0] == (2, 4, 1) and b2.shape == (2, 4, 1)
