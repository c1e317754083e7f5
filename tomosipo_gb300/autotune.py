"""Autotuner for the forward projector's launch schedule.

The forward projector runs its tiles (32 detector rows x 8 columns of one
pair of adjacent angles) in an order set by three numbers (``tsgb_tuning``):
detector patches of ``fp_patch_rows`` x ``fp_patch_cols`` tiles and groups of
``fp_group_pairs`` angle pairs. A group's tiles over one patch run together,
so the volume slab their rays cross stays in L2 across the group's angles. A
fourth, ``fp_pair_layout``, stores the padded volume copies as neighbour
pairs (two 8-byte loads per bilinear sample instead of four 4-byte ones, at
twice the footprint). The best values depend on the volume and detector
sizes and on the cone angle. ``autotune(A)`` times ``A``'s forward
projection under candidate settings with CUDA events (coordinate descent from
the default: element layout, patch rows, group size, patch columns, each from
the best so far) and sets the fastest on the operator's projector. The batched
SIRT solver launches each job's tiles in its projector's order, so tuning a
job's operator tunes its part of the batch.

Every schedule gives bit-identical results: only the order of independent
tiles changes. For operators with the matched backprojector the tuner then
times the backprojection under every kernel and warp shape it offers
(``bp_kernel``: voxel-pair threads or z-lane warps; ``bp_shape``: the z-lane
window x z run x warps per block) and sets the fastest; these change only the
order of fp32 sums. Results are cached per geometry (shapes, beam kind and a
hash of the projection vectors) in memory and, if ``cache_path`` is given, in a
JSON file. No counterpart in the reference, whose ASTRA launch shapes are
fixed.
"""
import hashlib
import json
import os

import torch

PAIR_LAYOUT = (0, 1)
PATCH_ROWS = (2, 4, 8, 16, 32)
GROUP_PAIRS = (8, 16, 32, 64, 128)
PATCH_COLS = (1, 2, 4, 8, 16)
# the order in which coordinate descent visits the settings
SEARCH = (("fp_pair_layout", PAIR_LAYOUT), ("fp_patch_rows", PATCH_ROWS),
          ("fp_group_pairs", GROUP_PAIRS), ("fp_patch_cols", PATCH_COLS))

# Matched backprojectors the tuner times: the voxel-pair kernel and every
# z-lane warp shape (include/tomosipo_gb300.h, tsgb_tuning.bp_shape).
BP_CANDIDATES = ({"bp_kernel": 0, "bp_shape": 0},) + tuple(
    {"bp_kernel": 1, "bp_shape": k} for k in range(7))

_cache = {}


def geometry_key(projector):
    """Stable key of a projector's geometry (shapes, kind, vectors)."""
    h = hashlib.sha1(projector._vectors.tobytes()).hexdigest()[:16]
    return "vol{}_sino{}_k{}_{}".format(
        "x".join(map(str, projector.vol_shape)),
        "x".join(map(str, projector.sino_shape)),
        int(projector.proj_desc.kind),
        h,
    )


def _load_file(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time_fp(A, x, y, repeats):
    """Mean CUDA-event time (ms) of ``repeats`` forward projections, after one warm-up."""
    A(x, out=y)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(repeats):
        A(x, out=y)
    end.record()
    end.synchronize()
    return start.elapsed_time(end) / repeats


def _time_bp(A, y, v, repeats):
    """Mean CUDA-event time (ms) of ``repeats`` backprojections, after one warm-up."""
    A.T(y, out=v)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(repeats):
        A.T(y, out=v)
    end.record()
    end.synchronize()
    return start.elapsed_time(end) / repeats


def fastest_candidate(start, candidates, measure):
    """Time ``start`` and then every other candidate (dicts of settings merged
    into ``start``); a candidate wins only if strictly faster. Returns
    ``(best, best_ms, start_ms, trials)``."""
    best = dict(start)
    best_ms = start_ms = measure(best)
    trials = 1
    for c in candidates:
        cand = dict(best, **c)
        if all(start.get(k) == v for k, v in c.items()):
            continue  # the starting point, already timed
        ms = measure(cand)
        trials += 1
        if ms < best_ms:
            best, best_ms = cand, ms
    return best, best_ms, start_ms, trials


def coordinate_descent(start, measure):
    """Coordinate descent over ``SEARCH`` from the settings ``start``.

    ``measure(tuning) -> ms`` times one candidate. Each setting in turn takes
    every listed value with the others fixed at the best so far; a candidate is
    kept only if strictly faster. Returns ``(best, best_ms, start_ms, trials)``.
    """
    best = dict(start)
    best_ms = measure(best)
    start_ms, trials = best_ms, 1
    for name, values in SEARCH:
        measured = best[name]  # this setting's value in the best point so far
        for v in values:
            if v == measured:
                continue
            cand = dict(best, **{name: v})
            ms = measure(cand)
            trials += 1
            if ms < best_ms:
                best, best_ms = cand, ms
    return best, best_ms, start_ms, trials


def shape_key(projector):
    """Key of a projector's sizes and beam kind only (angles and vectors ignored):
    operators that share it take the same schedule well."""
    return "vol{}_det{}x{}_k{}".format(
        "x".join(map(str, projector.vol_shape)), projector.sino_shape[0],
        projector.sino_shape[2], int(projector.proj_desc.kind))


def autotune(A, device=None, repeats=None, cache_path=None, verbose=False, key=None):
    """Pick the fastest forward schedule for operator ``A`` and set it.

    ``key``: cache key (default: ``geometry_key``, the exact geometry; pass
    ``shape_key(A.projector)`` to share results between operators of the same
    sizes). Returns ``{"tuning": {...}, "ms": best time, "default_ms": time of
    the starting schedule, "trials": n, "cached": bool}``.
    """
    proj = A.projector
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    key = key or geometry_key(proj)
    hit = _cache.get(key)
    if hit is None and cache_path and os.path.exists(cache_path):
        hit = _load_file(cache_path).get(key)
    if hit is not None:
        proj.set_tuning(dev.index, **hit["tuning"])
        _cache[key] = hit
        return dict(hit, cached=True)

    with torch.cuda.device(dev):
        g = torch.Generator(device="cpu").manual_seed(0)
        x = torch.rand(A.domain_shape, generator=g).to(dev)
        y = torch.empty(A.range_shape, device=dev)
        # about 20 ms of projection per candidate, at least one call
        first = _time_fp(A, x, y, 1)
        reps = repeats or max(1, min(8, int(20.0 / max(first, 1e-3))))

        def measure(tuning):
            proj.set_tuning(dev.index, **tuning)
            ms = _time_fp(A, x, y, reps)
            if verbose:
                print(f"autotune {key}: {tuning} {ms:.3f} ms")
            return ms

        best, best_ms, default_ms, trials = coordinate_descent(proj.get_tuning(dev.index),
                                                               measure)
        proj.set_tuning(dev.index, **best)
        result = {"tuning": best, "ms": best_ms, "default_ms": default_ms, "trials": trials}
        if getattr(A, "backprojector", None) == "matched":
            v = torch.empty(A.domain_shape, device=dev)
            first_bp = _time_bp(A, y, v, 1)
            reps_bp = repeats or max(1, min(8, int(20.0 / max(first_bp, 1e-3))))

            def measure_bp(tuning):
                proj.set_tuning(dev.index, **tuning)
                ms = _time_bp(A, y, v, reps_bp)
                if verbose:
                    print(f"autotune {key}: {tuning} BP {ms:.3f} ms")
                return ms

            best, bp_ms, bp_default_ms, bp_trials = fastest_candidate(best, BP_CANDIDATES,
                                                                      measure_bp)
            proj.set_tuning(dev.index, **best)
            result.update(tuning=best, bp_ms=bp_ms, bp_default_ms=bp_default_ms,
                          bp_trials=bp_trials)
    _cache[key] = result
    if cache_path:
        data = _load_file(cache_path)
        data[key] = result
        tmp = cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    return dict(result, cached=False)
