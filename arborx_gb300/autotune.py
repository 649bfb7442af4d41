"""Autotuner for the library's runtime knobs (abx_tuning_set).

Knobs change speed only, never results (every knob value is covered by the
parity tests): SPATIAL_BUCKET / NEAREST_BUCKET (largest subtree whose leaves
a query scans from the Morton-ordered leaf copy instead of descending) and
SORT_TOP_PASSES (digits sorted by passes before the run fix-up of the hybrid
sort).  The tuner runs coordinate descent: each knob in turn takes the
candidate value with the lowest median time of a caller-supplied step (a
sample of the real workload), the others held at their current best, until a
full round changes nothing.  Results can be cached in a JSON file under a
workload key and are applied with abx_tuning_set.

    best = autotune_queries(bvh, ax.nearest(sample_queries, 16))
"""

import json
import os

from . import _lib

KNOBS = {
    "NEAREST_BUCKET": [1, 2, 4, 8, 16],
    "SPATIAL_BUCKET": [1, 4, 8, 16, 32],
    "SORT_TOP_PASSES": [0, 3, 4],
}
DEFAULTS = {"NEAREST_BUCKET": 1, "SPATIAL_BUCKET": 8, "SORT_TOP_PASSES": 3}


def apply(settings):
    """Set every knob of `settings` in the library."""
    L = _lib.load()
    for name, value in settings.items():
        _lib.check(L.abx_tuning_set(name.encode(), int(value)))


def reset():
    _lib.check(_lib.load().abx_tuning_reset())


def coordinate_descent(knobs, time_fn, start=None, max_rounds=3):
    """Minimise time_fn(settings) over the grid `knobs` ({name: [values]}) by
    coordinate descent from `start`.  Returns (best settings, best time,
    number of evaluations).  time_fn is called once per distinct setting."""
    best = dict(start or {k: v[0] for k, v in knobs.items()})
    cache = {}

    def cost(setting):
        key = tuple(sorted(setting.items()))
        if key not in cache:
            cache[key] = float(time_fn(dict(setting)))
        return cache[key]

    best_t = cost(best)
    for _ in range(max_rounds):
        changed = False
        for name, values in knobs.items():
            for v in values:
                trial = dict(best)
                trial[name] = v
                t = cost(trial)
                if t < best_t:
                    best, best_t, changed = trial, t, True
        if not changed:
            break
    return best, best_t, len(cache)


def median_ms(step, repeats=5, warmup=1):
    """Median CUDA-event time of step() in milliseconds."""
    import torch

    for _ in range(warmup):
        step()
    times = []
    for _ in range(repeats):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def autotune_queries(tree, predicates, knobs=None, cache_path=None, key=None, repeats=5):
    """Tune the query knobs for queries like `predicates` on `tree` (a sample
    of the real batch).  Applies and returns the best settings."""
    from .bvh import Intersects, query

    if knobs is None:
        name = "SPATIAL_BUCKET" if isinstance(predicates, Intersects) else "NEAREST_BUCKET"
        knobs = {name: KNOBS[name]}
    if cache_path and key and os.path.exists(cache_path):
        with open(cache_path) as f:
            cached = json.load(f).get(key)
        if cached:
            apply(cached)
            return cached

    def time_fn(setting):
        apply(setting)
        return median_ms(lambda: query(tree, predicates), repeats=repeats)

    start = {k: DEFAULTS.get(k, v[0]) for k, v in knobs.items()}
    best, _, _ = coordinate_descent(knobs, time_fn, start=start)
    apply(best)
    if cache_path and key:
        data = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                data = json.load(f)
        data[key] = best
        with open(cache_path, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    return best
