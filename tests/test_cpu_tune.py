"""The autotuner's search and cache on the host: the timing of a candidate is
replaced by a model (no GPU), so the choice logic, the margin, the capacity
raise after overflows and the shape-keyed JSON cache are checked alone."""
import json

import numpy as np

from metakonga_gb300 import engine, scenes, tune


def _fake_time(costs, overflow=False):
    """A stand-in for tune._time: ms per step from a function of the tuning."""
    seen = []

    def f(sc, tuning, warm, steps):
        seen.append(dict(tuning))
        st = {"verlet_overflows": 5 if overflow else 0, "triangle_overflows": 0}
        return costs(tuning), st
    return f, seen


def test_shape_key_groups_by_octave_and_walls():
    a = scenes.settle_box(n_side=10)
    b = scenes.settle_box(n_side=10)
    c = scenes.settle_box(n_side=20)
    assert tune.shape_key(a) == tune.shape_key(b)
    assert tune.shape_key(a) != tune.shape_key(c)          # another particle-count octave
    assert "planes5" in tune.shape_key(a) and "tri0" in tune.shape_key(a)


def test_choice_needs_the_margin(monkeypatch, tmp_path):
    monkeypatch.setenv("XDEM_TUNE_CACHE", str(tmp_path / "t.json"))
    sc = scenes.settle_box(n_side=6)
    # skin 0.2 is 2 % faster (inside the 5 % margin), 128 threads 10 % faster
    def cost(t):
        c = 1.0
        if t["skin_factor"] == 0.2:
            c *= 0.98
        if t["contact_threads"] == 128:
            c *= 0.90
        return c
    f, seen = _fake_time(cost)
    monkeypatch.setattr(tune, "_time", f)
    out = tune.tune(sc, steps=10, warm=1)
    assert out["tuning"]["skin_factor"] == 0.1 and out["tuning"]["contact_threads"] == 128
    assert out["default_ms_per_step"] == 1.0 and abs(out["ms_per_step"] - 0.9) < 1e-12
    assert seen[0] == engine.DEFAULT_TUNING
    # cached under the scene's shape and read back
    cache = json.loads((tmp_path / "t.json").read_text())
    assert cache[tune.shape_key(sc)]["tuning"] == out["tuning"]
    assert tune.tuned(sc) == out["tuning"]
    # an unknown shape gets the defaults
    assert tune.tuned(scenes.settle_box(n_side=25)) == engine.DEFAULT_TUNING


def test_overflow_raises_the_capacity(monkeypatch, tmp_path):
    monkeypatch.setenv("XDEM_TUNE_CACHE", str(tmp_path / "t.json"))
    sc = scenes.settle_box(n_side=6)
    f, seen = _fake_time(lambda t: 1.0 if t["verlet_cap"] == 48 else 1.2, overflow=True)
    monkeypatch.setattr(tune, "_time", f)
    out = tune.tune(sc, steps=10, warm=1, store=False)
    # the larger list is kept although slower: the defaults' lists overflowed
    assert out["tuning"]["verlet_cap"] == 96
    assert all(c["tuning"]["verlet_cap"] == 96 for c in out["candidates"][1:])
    assert not (tmp_path / "t.json").exists()


def test_candidates_cover_skins_threads_and_pair_passes(monkeypatch, tmp_path):
    monkeypatch.setenv("XDEM_TUNE_CACHE", str(tmp_path / "t.json"))
    sc = scenes.settle_box(n_side=6)
    rng = np.random.Generator(np.random.MT19937(3))
    table = {}

    def cost(t):
        key = tuple(sorted(t.items()))
        if key not in table:
            table[key] = float(rng.uniform(0.5, 1.5))
        return table[key]
    f, seen = _fake_time(cost)
    monkeypatch.setattr(tune, "_time", f)
    out = tune.tune(sc, steps=10, warm=1, store=False)
    skins = {t["skin_factor"] for t in seen}
    threads = {t["contact_threads"] for t in seen}
    modes = {t["contact_mode"] for t in seen}
    assert skins == set(tune.SKINS) and threads == set(tune.THREADS) and modes == set(tune.MODES)
    # the choice is within the margin of the fastest candidate
    assert out["ms_per_step"] * (1 - 0.05) <= min(c["ms_per_step"] for c in out["candidates"]) + 1e-12
