"""The autotuner's coordinate search (host logic, no GPU): it finds the
optimum of a separable cost, skips schedules that cannot run, keeps the
start when nothing is at least min_gain faster, and the knob table only
names mrt_tuning fields with values the C ABI accepts."""
import pytest

from minotert_gb300 import autotune
from minotert_gb300._lib import MrtError, Tuning


def test_coordinate_search_finds_separable_optimum():
    want = {"a": 2, "b": 7, "c": 0}

    def measure(t):
        return 10.0 + sum(abs(t[k] - want[k]) for k in want)

    best, ms, results = autotune.coordinate_search(measure, {"a": 0, "b": 0, "c": 1},
                                                   {"a": [0, 1, 2, 3], "b": [0, 7, 9], "c": [1, 0]})
    assert best == want and ms == 10.0
    assert results[0]["tuning"] == {"a": 0, "b": 0, "c": 1}
    assert len({tuple(sorted(r["tuning"].items())) for r in results}) == len(results)  # each timed once


def test_coordinate_search_skips_refused_and_small_gains():
    def measure(t):
        if t["a"] == 1:
            return None  # refused schedule
        return {0: 100.0, 2: 99.8, 3: 90.0}[t["a"]] + (0.0 if t["b"] == 0 else 50.0)

    best, ms, _ = autotune.coordinate_search(measure, {"a": 0, "b": 0}, {"a": [1, 2], "b": [5]})
    assert best == {"a": 0, "b": 0} and ms == 100.0  # 99.8 is inside the 0.5 % margin
    best, ms, _ = autotune.coordinate_search(measure, {"a": 0, "b": 0}, {"a": [1, 2, 3]})
    assert best["a"] == 3 and ms == 90.0
    with pytest.raises(MrtError):
        autotune.coordinate_search(measure, {"a": 1, "b": 0}, {"a": [0]})


def test_knob_values_are_valid_tuning_fields():
    fields = {f for f, _ in Tuning._fields_}
    k = autotune.knobs(8, sort=True)
    assert set(k) <= fields
    assert all(0 <= v <= 64 for v in k["trace_blocks_per_sm"])
    assert set(k["dynamic_fetch"]) <= {0, 1, 2, 3} and set(k["tri_spread"]) <= set(range(16))
    assert all(1 <= v <= 32 for v in k["refill_min"]) and set(k["overlap_shadow"]) <= {0, 1}
    assert all(0 <= v <= 16 for v in k["tail_bounce"]) and set(k["tail_from_hits"]) <= {0, 1}
