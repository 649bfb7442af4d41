"""The reference's ordered ray traversal (ArborX_TreeTraversal.hpp:338-489)
restated step for step in the oracle, against the reference's own tree ray
tests and against the brute-force ordering this library reports.

The restatement shows one behaviour of the reference that this library does
not copy: when both children of a node miss the ray and the queue is empty,
the walk still descends into the nearer child (ties: the right one) and
reports the leaf it ends on, whose distance is +inf.  The rows here (and the
reference's own tests) hold only the leaves the ray hits."""

import numpy as np

from oracle import oracle as o
from tests.helpers import uniform_points


def test_restated_ordered_traversal_on_reference_cases(golden):
    """test/tstQueryTreeRay.cpp: rays along the diagonal of ten boxes, both
    ways, and the one-leaf tree."""
    g = golden["rays"]
    tree = o.OracleTree(np.asarray(g["tree_boxes"], np.float32), is_box=True)
    for c in g["tree_ordered"]:
        off, ind, dist = tree.ray_ordered(o.ray_normalize(np.asarray([c["ray"]], np.float32)))
        assert ind.tolist() == c["indices"]
        assert np.all(np.isfinite(dist)) and np.all(np.diff(dist) >= 0)
    one = g["single_leaf"]
    t1 = o.OracleTree(np.asarray([one["box"]], np.float32), is_box=True)
    off, ind, _ = t1.ray_ordered(o.ray_normalize(np.asarray(one["rays"], np.float32)))
    assert off.tolist() == one["offsets"] and ind.tolist() == one["indices"]


def _scene(leaves):
    lo = uniform_points(5000, 61)
    if leaves == "box":
        geom = np.concatenate([lo, lo + 0.01 + 0.02 * uniform_points(5000, 62)], axis=1)
    else:
        geom = lo
    rng = np.random.default_rng(63)
    org = rng.uniform(-0.2, 1.2, (1500, 3))
    d = rng.normal(size=(1500, 3))
    d[:150, 1:] = 0.0
    rays = o.ray_normalize(np.concatenate([org, d], axis=1).astype(np.float32))
    return geom, rays


def test_restated_ordered_traversal_equals_rows_up_to_ties_and_dead_ends():
    for leaves in ("box", "point"):
        geom, rays = _scene(leaves)
        tree = o.OracleTree(geom, is_box=leaves == "box")
        wo, wi, wd = tree.ray_ordered(rays)
        bo, bi, bd = o.ray_brute(geom, rays, ordered=True, is_box=leaves == "box")
        dead_ends = 0
        for q in range(len(rays)):
            i, d = wi[wo[q]:wo[q + 1]], wd[wo[q]:wo[q + 1]]
            miss = ~np.isfinite(d)
            if miss.any():
                # at most one, always the last report
                assert miss.sum() == 1 and miss[-1]
                dead_ends += 1
            i, d = i[~miss], d[~miss]
            assert np.all(np.diff(d) >= 0)  # reported by increasing distance
            order = np.lexsort((i, d + np.float32(0)))  # ties by value, -0 == +0
            assert np.array_equal(i[order], bi[bo[q]:bo[q + 1]])
            assert np.array_equal(d[order].view(np.int32), bd[bo[q]:bo[q + 1]].view(np.int32))
        assert dead_ends > 0


def test_restated_nearest_ray_traversal_equals_rows_up_to_ties():
    """nearest(Ray, k) by the reference's nearest traversal with
    distance(Ray, Box): the same distances, bit for bit, as the first k of
    the ordered rows; the indices differ only where the k-th distance is
    tied with the next hit (the reference keeps the first one it meets, the
    rows here the smaller value)."""
    for leaves in ("box", "point"):
        geom, rays = _scene(leaves)
        tree = o.OracleTree(geom, is_box=leaves == "box")
        bo, bi, bd = o.ray_brute(geom, rays, ordered=True, is_box=leaves == "box")
        for k in (1, 3, 8):
            no, ni, nd = tree.ray_nearest_arborx(rays, k)
            for q in range(len(rays)):
                row_i, row_d = bi[bo[q]:bo[q + 1]], bd[bo[q]:bo[q + 1]]
                got_i, got_d = ni[no[q]:no[q + 1]], nd[no[q]:no[q + 1]]
                assert np.array_equal(got_d + np.float32(0), row_d[:k] + np.float32(0))
                if sorted(got_i.tolist()) != sorted(row_i[:k].tolist()):
                    assert len(row_d) > k and row_d[k - 1] == row_d[k]
    # the one-leaf tree reports its leaf whatever the distance (:158-167);
    # the rows here hold hits only
    one = o.OracleTree(np.asarray([[0, 0, 0, 1, 1, 1]], np.float32), is_box=True)
    miss = o.ray_normalize(np.asarray([[4, 5, 6, 7, 8, 9]], np.float32))
    off, ind, dist = one.ray_nearest_arborx(miss, 1)
    assert off.tolist() == [0, 1] and ind.tolist() == [0] and dist[0] == np.inf
