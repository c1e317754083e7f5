"""Host logic of the forward projector's autotuner (``tomosipo_gb300.autotune``):
the coordinate-descent search on synthetic timings and the cache, with a fake
operator (no GPU)."""
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


def test_full_search_sets_and_caches_the_fastest_schedule(tmp_path, monkeypatch):
    """``autotune`` end to end with the timing faked and tensors kept on the
    CPU: it measures every candidate on the operator's projector, leaves the
    fastest set, returns it and writes it to the cache file."""
    import contextlib
    import types

    import torch

    target = dict(DEFAULT, fp_group_pairs=128, fp_patch_cols=1)
    cost = _separable_cost(target)

    class Operator(_FakeOperator):
        domain_shape, range_shape = (2, 3, 4), (5, 6, 7)

        def __call__(self, x, out=None):
            return out

    A = Operator()
    timed = []

    def fake_time(op, x, y, repeats):
        assert op is A and x.shape == A.domain_shape and y.shape == A.range_shape
        timed.append(dict(op.projector.tuning))
        return cost(op.projector.tuning)

    cpu_torch = types.SimpleNamespace(
        device=lambda *a: torch.device("cpu"), Generator=torch.Generator, rand=torch.rand,
        empty=lambda shape, device=None: torch.empty(shape),
        cuda=types.SimpleNamespace(device=lambda d: contextlib.nullcontext(),
                                   current_device=lambda: 0))
    monkeypatch.setattr(at, "torch", cpu_torch)
    monkeypatch.setattr(at, "_time_fp", fake_time)
    path = tmp_path / "tuning.json"
    at._cache.pop("fake-key", None)
    r = at.autotune(A, cache_path=str(path), key="fake-key")
    assert not r["cached"] and r["tuning"] == target and A.projector.tuning == target
    assert r["trials"] == 14 and len(timed) == 15  # the first call sizes the repeats
    assert r["ms"] == 10.0 and r["default_ms"] == cost(DEFAULT)
    assert json.loads(path.read_text())["fake-key"]["tuning"] == target
    at._cache.pop("fake-key", None)


def test_batch_tunes_once_per_job_shape(monkeypatch):
    """``sirt.autotune_jobs``: one autotuner run per (volume, detector, beam
    kind), whose schedule every operator of that shape then takes; operators
    that differ only in their angles share it."""
    import contextlib
    import types

    import torch

    from tomosipo_gb300 import sirt

    class Projector(_FakeProjector):
        def __init__(self, vol, rows, angles, cols, kind):
            super().__init__()
            self.vol_shape, self.sino_shape = vol, (rows, angles, cols)
            self.proj_desc = types.SimpleNamespace(kind=kind)

    ops = []
    for vol, rows, angles, cols, kind in [((8, 8, 8), 8, 30, 12, 1), ((8, 8, 8), 8, 90, 12, 1),
                                          ((8, 8, 8), 8, 30, 12, 0), ((16, 16, 16), 16, 30, 24, 1),
                                          ((8, 8, 8), 8, 60, 12, 1)]:
        A = _FakeOperator()
        A.projector = Projector(vol, rows, angles, cols, kind)
        ops.append(A)
    runs = []

    def fake_autotune(A, device_index, key):
        runs.append(key)
        return {"tuning": dict(DEFAULT, fp_patch_rows=PATCH[len(runs) - 1])}

    PATCH = (2, 4, 16)
    monkeypatch.setattr(at, "autotune", fake_autotune)
    monkeypatch.setattr(torch.cuda, "device", lambda d: contextlib.nullcontext())
    tuning = sirt.autotune_jobs(ops, torch.device("cuda", 0))
    assert len(runs) == len(set(runs)) == len(tuning) == 3
    rows = [A.projector.tuning["fp_patch_rows"] for A in ops]
    assert rows == [2, 2, 4, 16, 2]  # the three cone 8^3 jobs share the first run


def test_backprojector_search_times_every_candidate_once():
    """``fastest_candidate``: the starting backprojector is timed once, then
    every other kernel / shape; the fastest wins, ties keep the earlier."""
    start = dict(DEFAULT, bp_kernel=1, bp_shape=2)
    seen = []

    def measure(t):
        seen.append((t["bp_kernel"], t["bp_shape"]))
        return {(0, 0): 3.0, (1, 4): 1.0, (1, 2): 2.0}.get(seen[-1], 5.0)

    best, best_ms, start_ms, trials = at.fastest_candidate(start, at.BP_CANDIDATES, measure)
    assert (best["bp_kernel"], best["bp_shape"]) == (1, 4) and best_ms == 1.0 and start_ms == 2.0
    assert trials == len(at.BP_CANDIDATES) == len(seen) == len(set(seen))
    assert {k: best[k] for k in DEFAULT} == DEFAULT  # forward settings untouched
    # every candidate is a valid tuning: kernel 0 or 1, shape 0 .. 6
    assert all(c["bp_kernel"] in (0, 1) and 0 <= c["bp_shape"] <= 6 for c in at.BP_CANDIDATES)
