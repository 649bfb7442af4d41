"""KDOP bounding volumes on the GPU against the CPU oracle, bit-exact:
the point/box to KDOP conversion, intersects(KDOP) predicates on point and
box trees and on brute force, and trees over KDOP values (nodes bounded by
KDOPs) answering box and KDOP predicates.  Rows come out in the traversal
order of the reference (leaves in Morton order), checked against the
oracle's brute force reordered by the oracle tree's leaf order."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu

KS = [6, 14, 18, 26]


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def kdop_kind(ax, k):
    return {6: ax.KDOP6, 14: ax.KDOP14, 18: ax.KDOP18, 26: ax.KDOP26}[k]


def random_boxes(n, seed, size=0.05):
    rng = np.random.default_rng(seed)
    lo = rng.random((n, 3), dtype=np.float32)
    return np.concatenate([lo, lo + size * rng.random((n, 3), dtype=np.float32)], axis=1)


def cut_kdops(kd, seed, frac=0.3):
    """KDOPs narrowed on their non-axis directions (corners or edges cut off),
    so that they are not the KDOPs of their axis boxes."""
    nd = kd.shape[1] // 2
    out = kd.copy()
    if nd == 3:
        return out
    rng = np.random.default_rng(seed)
    mn, mx = out[:, 3:nd], out[:, nd + 3:]
    w = mx - mn
    mn += (frac * rng.random(mn.shape) * w).astype(np.float32)
    mx -= (frac * rng.random(mx.shape) * w).astype(np.float32)
    return out


def tree_order(geom, is_box):
    return o.OracleTree(geom, is_box=is_box).leaves["value"]


def check(ax, tree, preds, kind, want_off, want_ind):
    ind, off = ax.query(tree, ax.intersects(cuda(preds), kind))
    assert np.array_equal(host(off), want_off)
    assert np.array_equal(host(ind), want_ind)


@pytest.mark.parametrize("k", KS)
def test_kdop_from_geometry(ax, k):
    nd = k // 2
    pts = uniform_points(5000, 3) * 4 - 2
    boxes = random_boxes(5000, 4, size=0.5)
    boxes[::97, 0], boxes[::97, 3] = 1.0, 0.0  # inverted ranges stay empty
    for g, is_box in ((pts, False), (boxes, True)):
        got = host(ax.kdop_from(cuda(g), k))
        want = o.kdop_from_geometry(g, nd, is_box=is_box)
        assert np.array_equal(got.view(np.int32), want.view(np.int32))


def test_kdop_query_golden(ax, golden):
    """test/tstQueryTreeIntersectsKDOP.cpp:26-91."""
    t = golden["kdops"]["tree"]
    x = o.kdop_empty(9)
    for p in t["kdop18_expand"]:
        o.kdop_expand(x, p)
    pts = np.asarray(t["points"], np.float32)
    tree = ax.BVH(cuda(pts))
    ind, off = ax.query(tree, ax.intersects(cuda(x[None]), ax.KDOP18))
    assert host(off).tolist() == t["query"]["offsets"]
    assert sorted(host(ind).tolist()) == t["query"]["indices"]
    ind, off = ax.query(tree, ax.intersects(cuda(np.zeros((0, 18), np.float32)), ax.KDOP18))
    assert host(off).tolist() == t["empty"]["offsets"] and host(ind).size == 0


@pytest.mark.parametrize("k", KS)
@pytest.mark.parametrize("leaves", ["point", "box"])
def test_kdop_predicates_on_box_and_point_trees(ax, k, leaves):
    nd = k // 2
    n = 20000
    geom = uniform_points(n, 10) if leaves == "point" else random_boxes(n, 11)
    preds = cut_kdops(o.kdop_from_geometry(random_boxes(1500, 12, size=0.15), nd, is_box=True), 13)
    tree = ax.BVH(cuda(geom))
    off, ind = o.kdop_spatial_brute(geom, leaves, preds, k)
    want = o.in_tree_order(off, ind, tree_order(geom, leaves == "box"))
    check(ax, tree, preds, kdop_kind(ax, k), off, want)
    # buffered single pass and the unsorted query order give the same rows
    ind2, off2 = ax.query(tree, ax.intersects(cuda(preds), kdop_kind(ax, k)),
                          ax.TraversalPolicy(buffer_size=4, sort_predicates=False))
    assert np.array_equal(host(off2), off) and np.array_equal(host(ind2), want)
    # brute force: ascending values
    bf = ax.BruteForce(cuda(geom))
    ind3, off3 = ax.query(bf, ax.intersects(cuda(preds), kdop_kind(ax, k)))
    assert np.array_equal(host(off3), off) and np.array_equal(host(ind3), ind)


@pytest.mark.parametrize("k", KS)
def test_kdop_tree_values_and_predicates(ax, k):
    nd = k // 2
    n = 25000
    values = cut_kdops(o.kdop_from_geometry(random_boxes(n, 20), nd, is_box=True), 21)
    order = tree_order(o.kdop_axis_boxes(values), True)
    tree = ax.BVH(cuda(values), kind=kdop_kind(ax, k))
    assert tree.size() == n and tree.kind == kdop_kind(ax, k)
    qboxes = random_boxes(1500, 22, size=0.1)
    off, ind = o.kdop_spatial_brute(values, k, qboxes, "box")
    check(ax, tree, qboxes, ax.BOX, off, o.in_tree_order(off, ind, order))
    qk = cut_kdops(o.kdop_from_geometry(random_boxes(1500, 23, size=0.1), nd, is_box=True), 24)
    off, ind = o.kdop_spatial_brute(values, k, qk, k)
    check(ax, tree, qk, kdop_kind(ax, k), off, o.in_tree_order(off, ind, order))
    # the tree's KDOP is the union of the values
    kb = np.asarray(tree.kdop_bounds(), np.float32)
    assert np.array_equal(kb[:nd], values[:, :nd].min(0)) and np.array_equal(kb[nd:], values[:, nd:].max(0))


@pytest.mark.parametrize("n", [0, 1, 2, 3, 33, 1000])
def test_kdop_tree_small_sizes(ax, n):
    """Empty, one-leaf and small KDOP trees (buckets, single leaves)."""
    k, nd = 14, 7
    values = cut_kdops(o.kdop_from_geometry(random_boxes(max(n, 1), 30, size=0.3)[:n], nd, True), 31)
    tree = ax.BVH(cuda(values.reshape(n, 14)), kind=ax.KDOP14)
    qk = o.kdop_from_geometry(random_boxes(400, 32, size=0.3), nd, is_box=True)
    off, ind = o.kdop_spatial_brute(values.reshape(n, 14), k, qk, k)
    order = tree_order(o.kdop_axis_boxes(values.reshape(n, 14)), True) if n else np.zeros(0, np.int32)
    check(ax, tree, qk, ax.KDOP14, off, o.in_tree_order(off, ind, order) if n else ind)


def test_kdop_tree_one_pass_and_point_values(ax):
    """KDOPs of points (the reference's test trees convert their primitives,
    test/ArborXTest_LegacyTree.hpp:50-60) with enough queries for the sampled
    one-pass CRS."""
    k, nd = 18, 9
    pts = uniform_points(20000, 40)
    values = host(ax.kdop_from(cuda(pts), k))
    tree = ax.BVH(cuda(values), kind=ax.KDOP18)
    qboxes = random_boxes(70000, 41, size=0.03)
    off, ind = o.kdop_spatial_brute(pts, "point", qboxes, "box")  # same answers as a point tree
    order = tree_order(o.kdop_axis_boxes(values), True)
    check(ax, tree, qboxes, ax.BOX, off, o.in_tree_order(off, ind, order))


def test_kdop_tree_save_load(ax, tmp_path):
    values = cut_kdops(o.kdop_from_geometry(random_boxes(20000, 50), 13, True), 51)
    tree = ax.BVH(cuda(values), kind=ax.KDOP26)
    tree.save(tmp_path / "k.abx")
    loaded = ax.BVH.load(tmp_path / "k.abx")
    assert loaded.kind == ax.KDOP26 and loaded.kdop_bounds() == tree.kdop_bounds()
    qk = o.kdop_from_geometry(random_boxes(1000, 52, size=0.1), 13, True)
    a = ax.query(tree, ax.intersects(cuda(qk)))
    b = ax.query(loaded, ax.intersects(cuda(qk)))
    assert all(torch.equal(x, y) for x, y in zip(a, b))


def test_kdop_tree_refuses_other_queries(ax):
    values = o.kdop_from_geometry(random_boxes(100, 60), 7, True)
    tree = ax.BVH(cuda(values), kind=ax.KDOP14)
    q = uniform_points(10, 61)
    with pytest.raises(ax.AbxError):
        ax.query(tree, ax.nearest(cuda(q), 3))
    with pytest.raises(ax.AbxError):
        ax.query(tree, ax.make_intersects(cuda(q), 0.1))
    with pytest.raises(ax.AbxError):
        ax.query(tree, ax.intersects(cuda(o.kdop_from_geometry(random_boxes(5, 62), 9, True))))
    with pytest.raises(ax.AbxError):
        ax.query(tree, ax.ordered_intersects(cuda(np.ones((3, 6), np.float32))))


def test_kdop_predicates_on_a_forest(ax):
    """intersects(KDOP) over a batch of trees: each tree's rows equal those of
    the tree built alone (tree-local values)."""
    sizes = [0, 1, 500, 3000, 17]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    pts = uniform_points(int(off[-1]), 71)
    nqs = [5, 40, 300, 200, 3]
    qoff = np.concatenate([[0], np.cumsum(nqs)]).astype(np.int64)
    preds = cut_kdops(o.kdop_from_geometry(random_boxes(int(qoff[-1]), 72, size=0.2), 7, True), 73)
    forest = ax.Forest(cuda(pts), off)
    ind, got_off = forest.query(ax.intersects(cuda(preds), ax.KDOP14), qoff)
    ind, got_off = host(ind), host(got_off)
    for t in range(len(sizes)):
        tp = pts[off[t]:off[t + 1]]
        q = preds[qoff[t]:qoff[t + 1]]
        w_off, w_ind = o.kdop_spatial_brute(tp, "point", q, 14)
        if len(tp):
            w_ind = o.in_tree_order(w_off, w_ind, tree_order(tp, False))
        rows = got_off[qoff[t]:qoff[t + 1] + 1]
        assert np.array_equal(rows - rows[0], w_off)
        assert np.array_equal(ind[rows[0]:rows[-1]], w_ind)
