"""Batched trees (abx_forest_*): every tree of a forest equals the tree built
alone from its rows, bit for bit, and a forest query returns what the
per-tree queries return.  The per-tree form is the reference's many-trees
pattern (benchmarks/execution_space_instances/
execution_space_instances_driver.cpp:187-233)."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import cloud_box_queries, clouds, uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def bits(a):
    return np.asarray(a, np.float32).view(np.int32)


RAGGED = [0, 1, 2, 3, 17, 0, 100, 1000, 5000, 1, 257, 0]


def _same_nodes(forest, t, alone):
    fl, fi = forest.export_nodes(t)
    al, ai = alone.export_nodes()
    assert np.array_equal(fl.cpu().numpy(), al.cpu().numpy()), t
    assert np.array_equal(fi.cpu().numpy(), ai.cpu().numpy()), t
    assert np.array_equal(bits(forest.bounds(t)), bits(alone.bounds())), t


@pytest.mark.parametrize("kind", ["point", "box"])
def test_forest_trees_equal_trees_built_alone(ax, kind):
    pts, off, ext = clouds(RAGGED, 3)
    vals = pts if kind == "point" else cloud_box_queries(pts, off, ext, 0.05)
    forest = ax.Forest(cuda(vals), off)
    assert forest.num_trees() == len(RAGGED)
    for t, n in enumerate(RAGGED):
        assert forest.size(t) == n
        alone = ax.BoundingVolumeHierarchy(cuda(vals[off[t]:off[t + 1]]).reshape(-1, vals.shape[1]),
                                           kind=0 if kind == "point" else 1)
        _same_nodes(forest, t, alone)
    assert ax.device_errors() == 0


def test_forest_trees_equal_oracle(ax):
    """Against the CPU restatement directly (reference node layout)."""
    pts, off, _ = clouds([3000, 2, 777, 12000], 4)
    forest = ax.Forest(cuda(pts), off)
    for t in range(4):
        ref = o.OracleTree(pts[off[t]:off[t + 1]])
        leaves, internal = forest.export_nodes(t)
        leaves = leaves.cpu().numpy()
        assert np.array_equal(leaves[:, 0], ref.leaves["rope"])
        assert np.array_equal(leaves[:, 1], ref.leaves["value"])
        assert np.array_equal(internal.cpu().numpy(), ref.internal.view(np.int32).reshape(-1, 8))
        assert np.array_equal(bits(forest.bounds(t)), bits(ref.bounds))


def test_forest_of_duplicates_and_many_small_trees(ax):
    rng = np.random.default_rng(8)
    sizes = np.floor(10 ** rng.uniform(0, 3, 600)).astype(np.int64)
    sizes[::7] = 0
    pts, off, _ = clouds(sizes, 9)
    pts[off[5]:off[6]] = pts[off[5]]  # one tree of identical points
    forest = ax.Forest(cuda(pts), off)
    for t in list(range(0, 600, 37)) + [5]:
        alone = ax.BoundingVolumeHierarchy(cuda(pts[off[t]:off[t + 1]]).reshape(-1, 3))
        _same_nodes(forest, t, alone)


def _per_tree_crs(results, qoff):
    idx, offs = [], [0]
    for t, r in enumerate(results):
        i, o_ = r[0].cpu().numpy(), r[1].cpu().numpy()
        idx.append(i)
        offs.extend((o_[1:] + offs[-1]).tolist())
    return np.concatenate(idx) if idx else np.zeros(0, np.int32), np.asarray(offs, np.int32)


@pytest.mark.parametrize("sort", [True, False])
@pytest.mark.parametrize("buffer", [0, 4, -64])
def test_forest_box_queries_equal_per_tree_queries(ax, sort, buffer):
    pts, off, ext = clouds(RAGGED, 5)
    boxes = cloud_box_queries(pts, off, ext, 0.1)
    forest = ax.Forest(cuda(pts), off)
    pol = ax.TraversalPolicy().setPredicateSorting(sort).setBufferSize(buffer)
    fi, fo = forest.query(ax.intersects(cuda(boxes), kind=1), off, pol)
    per = []
    for t in range(len(RAGGED)):
        alone = ax.BoundingVolumeHierarchy(cuda(pts[off[t]:off[t + 1]]).reshape(-1, 3))
        per.append(ax.query(alone, ax.intersects(cuda(boxes[off[t]:off[t + 1]]).reshape(-1, 6), kind=1), pol))
    want_i, want_o = _per_tree_crs(per, off)
    assert np.array_equal(fo.cpu().numpy(), want_o)
    assert np.array_equal(fi.cpu().numpy(), want_i)
    # and against the oracle on one tree
    t = 8
    ref_o, ref_i = o.OracleTree(pts[off[t]:off[t + 1]]).spatial(o.KIND_BOX, boxes[off[t]:off[t + 1]])
    got_o = fo.cpu().numpy()[off[t]:off[t + 1] + 1]
    assert np.array_equal(got_o - got_o[0], ref_o)
    assert np.array_equal(fi.cpu().numpy()[got_o[0]:got_o[-1]], ref_i)


def test_forest_sphere_queries_with_uneven_query_counts(ax):
    pts, off, _ = clouds([500, 0, 2000, 64], 6)
    rng = np.random.default_rng(1)
    qsizes = [300, 5, 0, 1000]
    qoff = np.concatenate([[0], np.cumsum(qsizes)])
    spheres = []
    for t, m in enumerate(qsizes):
        lo, hi = off[t], off[t + 1]
        c = pts[lo:hi].mean(0) if hi > lo else np.zeros(3, np.float32)
        s = np.concatenate([c + rng.normal(0, 1, (m, 3)), rng.uniform(0, 0.5, (m, 1))], axis=1)
        spheres.append(s.astype(np.float32))
    spheres = np.concatenate(spheres)
    forest = ax.Forest(cuda(pts), off)
    fi, fo = forest.query(ax.intersects(cuda(spheres)), qoff)
    fo = fo.cpu().numpy()
    fi = fi.cpu().numpy()
    for t in range(4):
        ref = o.OracleTree(pts[off[t]:off[t + 1]])
        ro, ri = ref.spatial(o.KIND_SPHERE, spheres[qoff[t]:qoff[t + 1]])
        seg = fo[qoff[t]:qoff[t + 1] + 1]
        assert np.array_equal(seg - seg[0], ro)
        assert np.array_equal(fi[seg[0]:seg[-1]], ri)


@pytest.mark.parametrize("k", [1, 4, 16, 40])
def test_forest_nearest_equals_per_tree(ax, k):
    pts, off, _ = clouds(RAGGED, 7)
    q = uniform_points(int(off[-1]), 70) * 100
    forest = ax.Forest(cuda(pts), off)
    fi, fo, fd = forest.query(ax.nearest(cuda(q), k), off, with_distances=True)
    fo, fi, fd = fo.cpu().numpy(), fi.cpu().numpy(), fd.cpu().numpy()
    for t in range(len(RAGGED)):
        lo, hi = off[t], off[t + 1]
        ref = o.OracleTree(pts[lo:hi])
        ro, ri, rd = ref.nearest(q[lo:hi], k)
        seg = fo[lo:hi + 1]
        assert np.array_equal(seg - seg[0], ro), t
        assert np.array_equal(fi[seg[0]:seg[-1]], ri), t
        assert np.array_equal(bits(fd[seg[0]:seg[-1]]), bits(rd)), t


def test_forest_nearest_per_query_k(ax):
    pts, off, _ = clouds([50, 3, 0, 400], 11)
    rng = np.random.default_rng(2)
    q = (rng.random((int(off[-1]), 3)) * 100).astype(np.float32)
    kq = rng.integers(-2, 60, q.shape[0]).astype(np.int32)
    forest = ax.Forest(cuda(pts), off)
    fi, fo = forest.query(ax.nearest(cuda(q), cuda(kq)), off)
    fo, fi = fo.cpu().numpy(), fi.cpu().numpy()
    for t in range(4):
        lo, hi = off[t], off[t + 1]
        ro, ri, _ = o.OracleTree(pts[lo:hi]).nearest(q[lo:hi], kq[lo:hi])
        seg = fo[lo:hi + 1]
        assert np.array_equal(seg - seg[0], ro)
        assert np.array_equal(fi[seg[0]:seg[-1]], ri)


def test_single_tree_forest_equals_bvh(ax):
    p = uniform_points(200000, 12)
    forest = ax.Forest(cuda(p), [0, p.shape[0]])
    _same_nodes(forest, 0, ax.BoundingVolumeHierarchy(cuda(p)))
    q = uniform_points(5000, 13)
    a = forest.query(ax.nearest(cuda(q), 8), [0, 5000])
    b = ax.query(ax.BoundingVolumeHierarchy(cuda(p)), ax.nearest(cuda(q), 8))
    assert all(np.array_equal(x.cpu().numpy(), y.cpu().numpy()) for x, y in zip(a, b))


def test_forest_rejects_bad_offsets(ax):
    p = cuda(uniform_points(10, 1))
    with pytest.raises(ValueError):
        ax.Forest(p, [0, 5, 9])
    with pytest.raises(ax.SearchException):
        ax.Forest(p, [0, 6, 5, 10])
    forest = ax.Forest(p, [0, 4, 10])
    with pytest.raises(ValueError):
        forest.query(ax.nearest(p, 1), [0, 10])
    with pytest.raises(ax.SearchException):
        forest.query(ax.nearest(p, 1), [1, 4, 10])
