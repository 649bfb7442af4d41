"""BruteForce (src/spatial/ArborX_BruteForce.hpp:40-176): exact all-pairs
queries.  Nearest results equal the tree's and the oracle's bit for bit;
intersects results equal the oracle's brute force in ascending value order."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def bits(a):
    return np.asarray(a, np.float32).view(np.int32)


@pytest.mark.parametrize("k", [1, 5, 16, 32, 40])
def test_brute_nearest_equals_tree_and_oracle(ax, k):
    p = uniform_points(3000, 50)
    p[100:140] = p[100]  # exact ties
    q = uniform_points(777, 51)
    bf = ax.BruteForce(cuda(p))
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    bi, bo, bd = ax.query(bf, ax.nearest(cuda(q), k), with_distances=True)
    ti, to, td = ax.query(bvh, ax.nearest(cuda(q), k), with_distances=True)
    assert np.array_equal(bo.cpu().numpy(), to.cpu().numpy())
    assert np.array_equal(bi.cpu().numpy(), ti.cpu().numpy())
    assert np.array_equal(bits(bd.cpu().numpy()), bits(td.cpu().numpy()))
    ri, rd = o.knn_brute(p, q, k)
    assert np.array_equal(bi.cpu().numpy(), ri.ravel())
    assert np.array_equal(bits(bd.cpu().numpy()), bits(rd.ravel()))


def test_brute_nearest_per_query_k_and_boxes(ax):
    rng = np.random.default_rng(3)
    lo = uniform_points(2500, 52)
    b = np.concatenate([lo, lo + 0.01 * uniform_points(2500, 53)], axis=1)
    q = uniform_points(500, 54)
    kq = rng.integers(-1, 50, 500).astype(np.int32)
    bf = ax.BruteForce(cuda(b), kind=1)
    bvh = ax.BoundingVolumeHierarchy(cuda(b), kind=1)
    a = ax.query(bf, ax.nearest(cuda(q), cuda(kq)))
    t = ax.query(bvh, ax.nearest(cuda(q), cuda(kq)))
    assert all(np.array_equal(x.cpu().numpy(), y.cpu().numpy()) for x, y in zip(a, t))


@pytest.mark.parametrize("buffer", [0, 3, -1000])
def test_brute_spatial_equals_oracle(ax, buffer):
    p = uniform_points(5000, 55)
    rng = np.random.default_rng(4)
    sph = np.concatenate([uniform_points(1000, 56), rng.uniform(0, 0.08, (1000, 1))], axis=1).astype(np.float32)
    bf = ax.BruteForce(cuda(p))
    pol = ax.TraversalPolicy().setBufferSize(buffer)
    i, off = ax.query(bf, ax.intersects(cuda(sph)), pol)
    ro, ri = o.spatial_brute(p, o.KIND_SPHERE, sph)
    assert np.array_equal(off.cpu().numpy(), ro)
    assert np.array_equal(i.cpu().numpy(), ri)  # ascending value order
    boxes = np.concatenate([uniform_points(300, 57), uniform_points(300, 57) + 0.05], axis=1)
    i, off = ax.query(bf, ax.intersects(cuda(boxes)))
    ro, ri = o.spatial_brute(p, o.KIND_BOX, boxes)
    assert np.array_equal(off.cpu().numpy(), ro) and np.array_equal(i.cpu().numpy(), ri)


def test_brute_empty_and_bounds(ax):
    e = ax.BruteForce(torch.zeros((0, 3), device="cuda"))
    assert e.empty()
    i, off = ax.query(e, ax.nearest(cuda(uniform_points(4, 1)), 3))
    assert off.cpu().numpy().tolist() == [0] * 5 and i.numel() == 0
    p = uniform_points(100, 2)
    bf = ax.BruteForce(cuda(p))
    assert np.array_equal(bits(bf.bounds()), bits(np.concatenate([p.min(0), p.max(0)])))


@pytest.mark.parametrize("case", ["uniform", "duplicates", "far", "nonfinite", "clustered"])
@pytest.mark.parametrize("k", [1, 16, 32])
def test_tensor_filter_equals_plain_brute_force(ax, case, k):
    """The tensor-core candidate filter (BRUTE_TENSOR, Morton-ordered scan)
    returns exactly what the plain brute-force kernel returns: ties,
    duplicates, coordinates far from the origin (filter out of range),
    infinite points, tight clusters."""
    rng = np.random.default_rng({"uniform": 1, "duplicates": 2, "far": 3, "nonfinite": 4,
                                 "clustered": 5}[case])
    p = uniform_points(3000, 151)
    q = uniform_points(700, 152)
    if case == "duplicates":
        p = np.repeat(p[:300], 10, axis=0)
        q[::3] = p[::9][: len(q[::3])]
    elif case == "far":
        p = p * 1e16 + 3e16
        q = q * 1e16 + 3e16
    elif case == "nonfinite":
        # infinite points (their squared distances are inf or NaN: never
        # nearer than a finite point); queries with non-finite coordinates
        # have no defined answer (every distance is inf or NaN) and are left out
        p[::97] = np.inf
    elif case == "clustered":
        p = (0.5 + 1e-3 * rng.standard_normal((3000, 3))).astype(np.float32)
        q = (0.5 + 1e-3 * rng.standard_normal((700, 3))).astype(np.float32)
    L = ax._lib.load()
    bf = ax.BruteForce(cuda(p))
    scale = 1e16 if case == "far" else 1.0
    radius = np.float32(0.06 * scale if case != "clustered" else 3e-4)
    spheres = np.concatenate([q, np.full((len(q), 1), radius, np.float32)], axis=1)
    spheres[::7, 3] = -1.0  # negative radii match nothing
    try:
        ax._lib.check(L.abx_tuning_set(b"BRUTE_TENSOR", 1))
        a = ax.query(bf, ax.nearest(cuda(q), k), with_distances=True)
        sa = [ax.query(bf, ax.intersects(cuda(spheres)), ax.TraversalPolicy(buf))
              for buf in (0, 8, -64)] if k == 16 else []
        ax._lib.check(L.abx_tuning_set(b"BRUTE_TENSOR", 0))
        b = ax.query(bf, ax.nearest(cuda(q), k), with_distances=True)
        sb = [ax.query(bf, ax.intersects(cuda(spheres)), ax.TraversalPolicy(buf))
              for buf in (0, 8, -64)] if k == 16 else []
    finally:
        L.abx_tuning_reset()
    for x, y in zip(sa, sb):
        assert torch.equal(x[0], y[0]) and torch.equal(x[1], y[1])
    for x, y in zip(a, b):
        assert torch.equal(x.view(torch.int32) if x.dtype == torch.float32 else x,
                           y.view(torch.int32) if y.dtype == torch.float32 else y)
    if case == "uniform":
        bi, bd = o.knn_brute(p, q, k)
        assert np.array_equal(a[0].cpu().numpy().reshape(len(q), k), bi)
    assert ax.device_errors() == 0
