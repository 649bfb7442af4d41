"""Property tests of the CPU oracle on random small inputs (hypothesis):
its tree traversals agree with its brute force, KDOP tests are symmetric and
contain their own geometry, and half-to-full expansion gives symmetric lists.
No GPU needed."""

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings  # noqa: E402
from hypothesis import strategies as st  # noqa: E402

from oracle import oracle as o  # noqa: E402

coords = st.integers(min_value=0, max_value=8).map(lambda v: np.float32(v) / np.float32(8))


def point_sets(min_size=1, max_size=60):
    return st.lists(st.tuples(coords, coords, coords), min_size=min_size, max_size=max_size).map(
        lambda rows: np.asarray(rows, np.float32).reshape(-1, 3))


@settings(max_examples=60, deadline=None)
@given(point_sets(), point_sets(max_size=20), st.integers(min_value=1, max_value=12))
def test_tree_nearest_equals_brute_force(p, q, k):
    """Lattice points make ties common; the (distance, index) rule decides."""
    off, ind, dist = o.OracleTree(p).nearest(q, k)
    bi, bd = o.knn_brute(p, q, k)
    assert np.array_equal(ind, bi.ravel()) and np.array_equal(dist, bd.ravel())


@settings(max_examples=60, deadline=None)
@given(point_sets(), point_sets(max_size=20), st.integers(min_value=0, max_value=6))
def test_tree_spatial_equals_brute_force(p, q, r8):
    tree = o.OracleTree(p)
    spheres = np.concatenate([q, np.full((len(q), 1), np.float32(r8) / 8, np.float32)], axis=1)
    boxes = np.concatenate([q - np.float32(r8) / 16, q + np.float32(r8) / 16], axis=1)
    for kind, preds in ((o.KIND_SPHERE, spheres), (o.KIND_BOX, boxes)):
        off, ind = tree.spatial(kind, preds)
        boff, bind = o.spatial_brute(p, kind, preds)
        assert np.array_equal(off, boff)
        assert all(sorted(ind[off[i]:off[i + 1]]) == sorted(bind[boff[i]:boff[i + 1]])
                   for i in range(len(q)))


@settings(max_examples=80, deadline=None)
@given(point_sets(1, 6), point_sets(1, 6), st.sampled_from([3, 7, 9, 13]))
def test_kdop_tests_are_symmetric_and_contain_their_points(a, b, nd):
    ka, kb = o.kdop_empty(nd), o.kdop_empty(nd)
    for x in a:
        o.kdop_expand(ka, x)
    for x in b:
        o.kdop_expand(kb, x)
    assert o.kdop_intersects(ka, kb) == o.kdop_intersects(kb, ka)
    assert all(o.kdop_intersects(ka, x) for x in a)
    if any(o.kdop_intersects(kb, x) for x in a):
        assert o.kdop_intersects(ka, kb)


@settings(max_examples=60, deadline=None)
@given(st.integers(min_value=1, max_value=12).flatmap(
    lambda n: st.lists(st.lists(st.integers(min_value=0, max_value=n - 1), max_size=4),
                       min_size=n, max_size=n)))
def test_expand_half_to_full_is_symmetric(rows):
    off = [0]
    ind = []
    for r in rows:
        ind += r
        off.append(len(ind))
    foff, find = o.expand_half_to_full(off, ind)
    n = len(rows)
    full = [sorted(find[foff[i]:foff[i + 1]]) for i in range(n)]
    for i in range(n):
        for j in set(full[i]):
            assert full[j].count(i) == full[i].count(j)
    assert foff[-1] == 2 * len(ind)
