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
