"""The launch-shape autotuner's host side: the coordinate-descent search, the
tuning table behind mt_tuning_get / mt_tuning_set (no GPU needed) and the JSON a
search persists."""
import json

import pytest

from mambatracer_gb300 import api, tune
from mambatracer_gb300._lib import MTError


def test_search_finds_the_best_of_a_separable_score():
    space = {"a": (1, 2, 3), "b": (10, 20, 30), "c": (0, 5)}
    best_of = {"a": 3, "b": 20, "c": 5}
    calls = []

    def measure(t):
        calls.append(dict(t))
        return -sum(abs(t[k] - best_of[k]) for k in space)

    best, score, trials = tune.search(measure, {"a": 1, "b": 10, "c": 0}, space, rounds=3)
    assert best == best_of and score == 0
    assert len(trials) == len(calls)  # each tuning measured once
    assert len({tuple(sorted(t.items())) for t in calls}) == len(calls)


def test_search_keeps_the_start_when_nothing_beats_it():
    space = {"a": (1, 2), "b": (3, 4)}
    best, score, trials = tune.search(lambda t: 1.0 if t == {"a": 1, "b": 3} else 0.5, {"a": 1, "b": 3}, space)
    assert best == {"a": 1, "b": 3} and score == 1.0 and len(trials) == 3


def test_tuning_table_round_trip_and_range_checks():
    before = api.get_tuning()
    assert set(before) == set(tune.SPACE)
    try:
        api.set_tuning(closest_minb=8, shadow_minb=16, closest_grid=3, shadow_grid=0, shade_minb=5, refill_steps=32,
                       shadow_stream=1)
        assert api.get_tuning() == {"closest_minb": 8, "shadow_minb": 16, "closest_grid": 3, "shadow_grid": 0,
                                    "shade_minb": 5, "refill_steps": 32, "shadow_stream": 1}
        for bad in ({"closest_minb": 10}, {"shadow_minb": 4}, {"closest_grid": 33}, {"shadow_grid": -1},
                    {"shade_minb": 6}, {"refill_steps": 2}, {"refill_steps": 2048}, {"shadow_stream": 2}):
            with pytest.raises(MTError, match="out of range"):
                api.set_tuning(bad)
        assert api.get_tuning()["closest_minb"] == 8  # a refused tuning leaves the table alone
    finally:
        api.set_tuning(before)
    assert api.get_tuning() == before


def test_persisted_tuning_loads_only_on_a_matching_device(tmp_path, monkeypatch):
    before = api.get_tuning()
    dev = {"name": "a GPU", "sms": 152}
    monkeypatch.setattr(tune, "device_info", lambda device=0: dict(dev))
    res = {"device": dict(dev), "workload": "w", "tuning": dict(before, refill_steps=128), "mrays_per_s": 1.0,
           "start": {"tuning": before, "mrays_per_s": 0.9}, "trials": []}
    path = tmp_path / "t.json"
    tune.save(str(path), res)
    assert json.loads(path.read_text()) == res
    try:
        assert tune.load(str(path)) == res and api.get_tuning()["refill_steps"] == 128
        api.set_tuning(before)
        dev["sms"] = 148
        assert tune.load(str(path)) is None and api.get_tuning() == before
        assert tune.load(str(path), require_match=False) == res and api.get_tuning()["refill_steps"] == 128
    finally:
        api.set_tuning(before)


def test_search_ignores_gains_inside_the_noise_and_confirms_the_winner():
    space = {"a": (1, 2, 3)}
    # a=2 scores 0.5 % above the start: inside min_gain, never adopted
    best, _, _ = tune.search(lambda t: {1: 100.0, 2: 100.5, 3: 99.0}[t["a"]], {"a": 1}, space, min_gain=0.01)
    assert best == {"a": 1}
    # a=3 looks 5 % better once, but not when measured again: the start is kept
    seen = {"n": 0}

    def flaky(t):
        if t["a"] == 3:
            seen["n"] += 1
            return 105.0 if seen["n"] == 1 else 99.0
        return 100.0

    best, score, trials = tune.search(flaky, {"a": 1}, space, min_gain=0.01, confirm=2)
    assert best == {"a": 1} and score == 100.0 and seen["n"] == 3
    # a real gain survives the confirmation
    best, score, _ = tune.search(lambda t: 100.0 + 3 * (t["a"] == 3), {"a": 1}, space, min_gain=0.01, confirm=2)
    assert best == {"a": 3} and score == 103.0


def test_bench_installs_shapes_only_for_their_workload_and_device(tmp_path, monkeypatch):
    import bench
    before = api.get_tuning()
    dev = {"name": "a GPU", "sms": 152}
    monkeypatch.setattr(tune, "device_info", lambda device=0: dict(dev))
    path = tmp_path / "tuning.json"
    tune.save(str(path), {"device": dict(dev), "workload": "the soup", "workload_key": "soup1000000_1920x1080",
                          "tuning": dict(before, refill_steps=32), "mrays_per_s": 1.0, "start": {}, "trials": []})
    monkeypatch.setattr(bench, "TUNED", str(path))
    try:
        assert bench.apply_tuning(None)["source"] == "built-in defaults"
        assert bench.apply_tuning("stadium3310720_1920x1080")["source"] == "built-in defaults"
        assert api.get_tuning() == before
        got = bench.apply_tuning("soup1000000_1920x1080")
        assert got["source"].startswith("autotuned") and got["tuning"]["refill_steps"] == 32
        api.set_tuning(before)
        dev["sms"] = 148  # another GPU model
        assert bench.apply_tuning("soup1000000_1920x1080")["source"] == "built-in defaults"
    finally:
        api.set_tuning(before)
