"""Rays (src/geometry/ArborX_Ray.hpp; ordered traversal
ArborX_TreeTraversal.hpp:338-489): the reference's tree ray tests
(test/tstQueryTreeRay.cpp), then random boxes and points against the
brute-force restatement: intersects(Ray) as a set in depth-first order,
ordered_intersects(Ray) exactly (indices and distances, ties by index)."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def rows(off, ind):
    off = off.cpu().numpy()
    ind = ind.cpu().numpy()
    return [ind[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


def test_reference_tree_ray_cases(ax, golden):
    g = golden["rays"]
    boxes = ax.BoundingVolumeHierarchy(cuda(g["tree_boxes"]), kind=ax.BOX)
    r = cuda([g["tree_intersects"]["ray"]])
    ind, off = ax.query(boxes, ax.ray_intersects(r))
    assert sorted(ind.cpu().numpy().tolist()) == g["tree_intersects"]["indices"]
    for c in g["tree_ordered"]:
        ind, off = ax.query(boxes, ax.ordered_intersects(cuda([c["ray"]])))
        assert ind.cpu().numpy().tolist() == c["indices"]
    nn = g["tree_nearest"]
    ind, off = ax.query(boxes, ax.ordered_intersects(cuda([nn["ray"]]), k=nn["k"]))
    assert ind.cpu().numpy().tolist() == nn["indices"]
    one = g["single_leaf"]
    t = ax.BoundingVolumeHierarchy(cuda([one["box"]]), kind=ax.BOX)
    ind, off = ax.query(t, ax.ordered_intersects(cuda(one["rays"])))
    assert off.cpu().numpy().tolist() == one["offsets"] and ind.cpu().numpy().tolist() == one["indices"]
    empty = ax.BoundingVolumeHierarchy(torch.zeros((0, 6), device="cuda"), kind=ax.BOX)
    ind, off = ax.query(empty, ax.ordered_intersects(cuda(one["rays"])))
    assert off.cpu().numpy().tolist() == [0, 0, 0]


def _random_rays(m, seed):
    rng = np.random.default_rng(seed)
    org = rng.uniform(-0.2, 1.2, (m, 3))
    d = rng.normal(size=(m, 3))
    d[:m // 10, 1:] = 0.0  # axis-aligned rays (zero direction components)
    return np.concatenate([org, d], axis=1).astype(np.float32)


@pytest.mark.parametrize("leaves", ["box", "point"])
def test_rays_against_brute_force(ax, leaves):
    lo = uniform_points(20000, 31)
    if leaves == "box":
        geom = np.concatenate([lo, lo + 0.01 + 0.02 * uniform_points(20000, 32)], axis=1)
        tree = ax.BoundingVolumeHierarchy(cuda(geom), kind=ax.BOX)
    else:
        geom = lo
        tree = ax.BoundingVolumeHierarchy(cuda(geom))
    rays = _random_rays(3000, 33)
    nrm = o.ray_normalize(rays)
    ro, ri, rd = o.ray_brute(geom, nrm, ordered=False, is_box=leaves == "box")
    ind, off = ax.query(tree, ax.ray_intersects(cuda(rays)))
    assert np.array_equal(off.cpu().numpy(), ro)
    assert [sorted(r) for r in rows(off, ind)] == rows(torch.from_numpy(ro), torch.from_numpy(ri))
    ro, ri, rd = o.ray_brute(geom, nrm, ordered=True, is_box=leaves == "box")
    ind, off, dist = ax.query(tree, ax.ordered_intersects(cuda(rays)), with_distances=True)
    assert np.array_equal(off.cpu().numpy(), ro)
    assert np.array_equal(ind.cpu().numpy(), ri)
    assert np.array_equal(dist.cpu().numpy().view(np.int32), rd.view(np.int32))
    # nearest(Ray, k): the first k of each ordered row
    ind, off = ax.query(tree, ax.ordered_intersects(cuda(rays), k=3))
    want = [r[:3] for r in rows(torch.from_numpy(ro), torch.from_numpy(ri))]
    assert rows(off, ind) == want
    assert ax.device_errors() == 0


def _ray_nearest_scene(leaves):
    """20000 leaves with 100 copies of one leaf (equal distances: ties go by
    index) and 3000 rays, the first 64 starting on a leaf's upper corner with
    every direction component negative, so that their entry distance into
    that leaf is -0."""
    lo = uniform_points(20000, 41)
    if leaves == "box":
        geom = np.concatenate([lo, lo + 0.01 + 0.02 * uniform_points(20000, 42)], axis=1)
    else:
        geom = lo.copy()
    geom[100:200] = geom[50]
    rays = _random_rays(3000, 43)
    corner = geom[:64, 3:6] if leaves == "box" else geom[:64, :3]
    rays[:64, :3] = corner
    rays[:64, 3:6] = -np.abs(rays[:64, 3:6]) - 0.1
    return geom, rays


@pytest.mark.parametrize("leaves", ["box", "point"])
@pytest.mark.parametrize("k", [1, 2, 5, 16, 32, 40])
def test_nearest_rays_pruned_walk(ax, leaves, k):
    """nearest(Ray, k) (a pruned walk for k <= 32) gives the first k entries
    of each ordered_intersects row: indices and distance bits, -0 included,
    equal to the oracle's and to the rows of the full ordering pass."""
    geom, rays = _ray_nearest_scene(leaves)
    tree = (ax.BoundingVolumeHierarchy(cuda(geom), kind=ax.BOX) if leaves == "box"
            else ax.BoundingVolumeHierarchy(cuda(geom)))
    ro, ri, rd = o.ray_brute(geom, o.ray_normalize(rays), ordered=True, is_box=leaves == "box")
    want_i = [ri[ro[q]:ro[q + 1]][:k].tolist() for q in range(len(rays))]
    want_d = [rd[ro[q]:ro[q + 1]][:k].view(np.int32).tolist() for q in range(len(rays))]
    assert any(np.signbit(rd[ro[q]]) for q in range(64) if ro[q + 1] > ro[q])
    ind, off, dist = ax.query(tree, ax.ordered_intersects(cuda(rays), k=k), with_distances=True)
    assert rows(off, ind) == want_i
    assert rows(off, dist.view(torch.int32)) == want_d
    # the same rows from the ordering pass, and without the distances
    L = ax._lib.load()
    try:
        ax._lib.check(L.abx_tuning_set(b"RAY_NEAREST", 0))
        ind0, off0, dist0 = ax.query(tree, ax.ordered_intersects(cuda(rays), k=k),
                                     with_distances=True)
    finally:
        L.abx_tuning_reset()
    assert torch.equal(off0, off) and torch.equal(ind0, ind)
    assert torch.equal(dist0.view(torch.int32), dist.view(torch.int32))
    ind1, off1 = ax.query(tree, ax.ordered_intersects(cuda(rays), k=k),
                          ax.TraversalPolicy(sort_predicates=False))
    assert torch.equal(off1, off) and torch.equal(ind1, ind)
    assert ax.device_errors() == 0


@pytest.mark.parametrize("n", [1, 2, 3, 40])
def test_nearest_rays_small_trees(ax, n):
    """One-leaf and small trees; rays that miss everything get empty rows."""
    geom = np.concatenate([uniform_points(n, 50), uniform_points(n, 50) + 0.2], axis=1)
    tree = ax.BoundingVolumeHierarchy(cuda(geom), kind=ax.BOX)
    rays = _random_rays(500, 51)
    ro, ri, _ = o.ray_brute(geom, o.ray_normalize(rays), ordered=True, is_box=True)
    for k in (1, 3):
        ind, off = ax.query(tree, ax.ordered_intersects(cuda(rays), k=k))
        assert rows(off, ind) == [ri[ro[q]:ro[q + 1]][:k].tolist() for q in range(len(rays))]
    assert ax.device_errors() == 0
