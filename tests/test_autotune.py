"""Autotuner: coordinate descent over the runtime knobs (host logic on the
CPU with a synthetic cost; the GPU test tunes a real query and checks that
results are unchanged)."""

import numpy as np
import pytest


def test_coordinate_descent_finds_the_grid_minimum():
    from arborx_gb300.autotune import coordinate_descent

    knobs = {"A": [1, 2, 4, 8, 16], "B": [0, 3]}
    calls = []

    def cost(s):
        calls.append(dict(s))
        return (np.log2(s["A"]) - 3) ** 2 + (0.5 if s["B"] == 0 else 0.0)

    best, t, evals = coordinate_descent(knobs, cost, start={"A": 1, "B": 0})
    assert best == {"A": 8, "B": 3} and t == 0.0
    assert evals == len({tuple(sorted(c.items())) for c in calls}) <= 5 * 2


def test_coordinate_descent_keeps_start_when_nothing_is_better():
    from arborx_gb300.autotune import coordinate_descent

    best, t, evals = coordinate_descent({"A": [1, 2, 3]}, lambda s: 1.0, start={"A": 2})
    assert best == {"A": 2} and evals == 3


@pytest.mark.gpu
def test_autotune_query_keeps_results(ax, tmp_path):
    import torch

    from arborx_gb300 import autotune
    from tests.helpers import uniform_points

    p = torch.from_numpy(uniform_points(200000, 60)).cuda()
    q = torch.from_numpy(uniform_points(50000, 61)).cuda()
    bvh = ax.BoundingVolumeHierarchy(p)
    before = [x.cpu().numpy() for x in ax.query(bvh, ax.nearest(q, 16))]
    try:
        best = autotune.autotune_queries(bvh, ax.nearest(q, 16), cache_path=str(tmp_path / "t.json"),
                                         key="knn16", repeats=3)
        assert set(best) == {"NEAREST_BUCKET"}
        after = [x.cpu().numpy() for x in ax.query(bvh, ax.nearest(q, 16))]
        assert all(np.array_equal(a, b) for a, b in zip(before, after))
        again = autotune.autotune_queries(bvh, ax.nearest(q, 16), cache_path=str(tmp_path / "t.json"),
                                          key="knn16")
        assert again == best  # from the cache
    finally:
        autotune.reset()
