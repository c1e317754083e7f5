"""Host logic of the forward projector's autotuner (``tomosipo_gb300.autotune``):
the coordinate-descent search on synthetic timings and the cache, with a fake
operator (no GPU)."""
import itertools
import json

import pytest

from tomosipo_gb300 import autotune as at

DEFAULT = {"fp_pair_layout": 0, "fp_patch_rows": 8, "fp_group_pairs": 32, "fp_patch_cols": 4}


def _separable_cost(target):
    """A timing that is smallest at ``target`` and adds one term per setting."""
    def measure(t):
        return 10.0 + sum(abs(_rank(k, t[k]) - _rank(k, target[k])) for k in t)
    return measure


def _rank(name, value):
    return dict(at.SEARCH)[name].index(value)


def test_descent_finds_the_minimum_of_a_separable_timing():
    for target in ({"fp_pair_layout": 1, "fp_patch_rows": 32, "fp_group_pairs": 8,
                    "fp_patch_cols": 16}, DEFAULT):
        best, best_ms, start_ms, trials = at.coordinate_descent(DEFAULT, _separable_cost(target))
        assert best == target and best_ms == 10.0 and start_ms >= best_ms
        # every other value of every setting once, plus the starting point
        assert trials == 1 + sum(len(values) - 1 for _, values in at.SEARCH) == 14


@pytest.mark.parametrize("moving", [False, True])
def test_descent_measures_no_candidate_twice_and_keeps_ties(moving):
    seen = []
    target = dict(DEFAULT, fp_patch_rows=2, fp_patch_cols=16)
    cost = _separable_cost(target)

    def measure(t):
        seen.append(tuple(sorted(t.items())))
        # flat: every schedule equally fast, so the start must survive
        return cost(t) if moving else 5.0

    best, best_ms, start_ms, trials = at.coordinate_descent(DEFAULT, measure)
    assert best == (target if moving else DEFAULT)
    assert len(seen) == len(set(seen)) == trials == 14


def test_descent_visits_settings_in_order_from_the_best_so_far():
    # Cheaper with the pair layout; patch rows only matter once it is set.
    def measure(t):
        return (1.0 if t["fp_pair_layout"] else 2.0) - (0.5 if t["fp_pair_layout"] and
                                                        t["fp_patch_rows"] == 2 else 0.0)

    best, best_ms, _, _ = at.coordinate_descent(DEFAULT, measure)
    assert best["fp_pair_layout"] == 1 and best["fp_patch_rows"] == 2 and best_ms == 0.5


class _FakeProjector:
    def __init__(self):
        self.tuning = dict(DEFAULT)

    def set_tuning(self, device_index, **values):
        self.tuning.update(values)

    def get_tuning(self, device_index=None):
        return dict(self.tuning)


class _FakeOperator:
    def __init__(self):
        self.projector = _FakeProjector()


def test_cache_file_serves_a_stored_schedule(tmp_path):
    stored = {"tuning": dict(DEFAULT, fp_patch_rows=16), "ms": 1.0, "default_ms": 2.0,
              "trials": 14}
    path = tmp_path / "tuning.json"
    path.write_text(json.dumps({"geometry-key": stored}))
    at._cache.pop("geometry-key", None)
    A = _FakeOperator()
    r = at.autotune(A, device=0, cache_path=str(path), key="geometry-key")
    assert r["cached"] and r["tuning"] == stored["tuning"]
    assert A.projector.tuning == stored["tuning"]
    B = _FakeOperator()  # now served from memory, without the file
    assert at.autotune(B, device=0, key="geometry-key")["cached"]
    assert B.projector.tuning == stored["tuning"]
    at._cache.pop("geometry-key", None)


@pytest.mark.parametrize("name, values", at.SEARCH)
def test_search_values_are_valid_tunings(name, values):
    assert len(set(values)) == len(values) and all(v >= 0 for v in values)
    assert DEFAULT[name] in values
