"""The autotuner's host logic (no GPU): size buckets, cache keys, the cache file
and the coordinate descent over launch parameters."""
import json

from diso_gb300 import tune


def test_buckets():
    assert tune.bucket((20, 20, 20)) == "n32"
    assert tune.bucket((64, 33, 10)) == "n64"
    assert tune.bucket((65, 2, 2)) == "n128"
    assert tune.bucket((512, 512, 512)) == "n512"


def test_coordinate_descent_finds_the_best_setting_one_parameter_at_a_time():
    # separable cost: each parameter's best value is found independently
    target = {"count_ctas": 1, "emit_ctas": 3, "fused_ctas": 0}
    calls = []

    def measure(s):
        calls.append(s)
        return sum((s[p] - target[p]) ** 2 for p in target) + 1.0

    best, t, seen = tune.coordinate_descent(list(target), tune.CANDIDATES, measure)
    assert best == target and t == 1.0
    # every setting is timed once: the default plus each other candidate of each parameter
    assert len(calls) == len(seen) == 1 + sum(len([v for v in tune.CANDIDATES[p] if v != 0]) for p in target)


def test_coordinate_descent_keeps_the_default_when_nothing_is_faster():
    best, t, _ = tune.coordinate_descent(["emit_ctas"], tune.CANDIDATES, lambda s: 1.0 + s["emit_ctas"])
    assert best == {"emit_ctas": 0} and t == 1.0


def test_cache_round_trip(tmp_path, monkeypatch):
    path = str(tmp_path / "sub" / "tune.json")
    monkeypatch.setenv("DISO_TUNE_CACHE", path)
    assert tune.cache_path() == path and tune.load_cache() == {}
    tune.store("a|dmc|float32|n512|recompute", {"params": {"emit_ctas": 2}, "ms": 1.0})
    tune.store("b|mc|float64|n64|stored", {"params": {}, "ms": 2.0})
    data = json.load(open(path))
    assert data["a|dmc|float32|n512|recompute"]["params"] == {"emit_ctas": 2} and len(data) == 2
    with open(path, "w") as f:
        f.write("not json")
    assert tune.load_cache() == {}


def test_every_parameter_is_a_library_parameter():
    from diso_gb300 import _native as N

    assert set(tune.CANDIDATES) == set(N.TUNE_PARAMS)
    for params in tune.MODE_PARAMS.values():
        assert set(params) <= set(tune.CANDIDATES)
        assert all(0 in tune.CANDIDATES[p] for p in params)  # the default is always a candidate
