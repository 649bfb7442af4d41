"""Trees written to disk and read back (abx_bvh_save / abx_bvh_load): the
loaded tree answers nearest and spatial queries bit-exactly like the oracle,
for points and boxes, for empty and one-leaf trees."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("n", [0, 1, 2, 1000, 200003])
def test_saved_point_tree_answers_like_the_oracle(ax, tmp_path, n):
    pts = uniform_points(n, 11)
    qs = uniform_points(3000, 12)
    path = tmp_path / "tree.abx"
    ax.BVH(cuda(pts)).save(path)
    tree = ax.BVH.load(path)
    assert tree.size() == n
    assert np.array_equal(np.asarray(tree.bounds(), np.float32).view(np.int32),
                          o.scene_bounds(pts).view(np.int32)) or n == 0
    ref = o.OracleTree(pts)
    ind, off, dist = ax.query(tree, ax.nearest(cuda(qs), 7), with_distances=True)
    r_off, r_ind, r_dist = ref.nearest(qs, 7)
    assert np.array_equal(off.cpu().numpy(), r_off)
    assert np.array_equal(ind.cpu().numpy(), r_ind)
    assert np.array_equal(dist.cpu().numpy().view(np.int32), r_dist.view(np.int32))
    spheres = np.concatenate([qs, np.full((len(qs), 1), 0.05, np.float32)], axis=1)
    ind, off = ax.query(tree, ax.intersects(cuda(spheres)))
    r_off, r_ind = ref.spatial(o.KIND_SPHERE, spheres)
    assert np.array_equal(off.cpu().numpy(), r_off)
    got = ind.cpu().numpy()
    for q in range(len(qs)):
        a, b = r_off[q], r_off[q + 1]
        assert np.array_equal(np.sort(got[a:b]), np.sort(r_ind[a:b]))

def test_saved_box_tree_matches_the_built_one(ax, tmp_path):
    lo = uniform_points(50000, 21)
    boxes = np.concatenate([lo, lo + 0.01], axis=1)
    qs = uniform_points(2000, 22)
    built = ax.BVH(cuda(boxes), kind=1)
    built.save(tmp_path / "boxes.abx")
    loaded = ax.BVH.load(tmp_path / "boxes.abx")
    assert loaded.kind == 1
    a = ax.query(built, ax.nearest(cuda(qs), 5), with_distances=True)
    b = ax.query(loaded, ax.nearest(cuda(qs), 5), with_distances=True)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    assert (tmp_path / "boxes.abx").stat().st_size == 48 + 49999 * 64 + 50000 * 32
