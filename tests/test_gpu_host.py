"""nearest(point, k) with host queries and host results
(abx_bvh_query_nearest_host): chunked, pipelined copies give exactly the
device query's CRS for every chunk size, k (register list and heap paths),
pinned and pageable buffers."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("chunk", [0, 1, 7, 1000, 4999, 5000, 100000])
@pytest.mark.parametrize("k", [1, 16, 40])
def test_host_nearest_equals_device_query(ax, chunk, k):
    p = uniform_points(30000, 141)
    q = uniform_points(5000, 142)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), k), with_distances=True)
    pin = chunk % 2 == 0
    qh = torch.from_numpy(q).pin_memory() if pin else torch.from_numpy(q)
    oh = torch.empty(len(q) + 1, dtype=torch.int32, pin_memory=pin)
    ih = torch.empty(len(q) * k, dtype=torch.int32, pin_memory=pin)
    dh = torch.empty(len(q) * k, dtype=torch.float32, pin_memory=pin)
    ax.query_nearest_host(bvh, qh, k, oh, ih, dh, chunk=chunk)
    assert torch.equal(oh, off.cpu()) and torch.equal(ih, ind.cpu())
    assert torch.equal(dh.view(torch.int32), dist.cpu().view(torch.int32))
    if k == 16 and chunk == 1000:
        roff, rind, _ = o.OracleTree(p).nearest(q, k)
        assert np.array_equal(ih.numpy(), rind)


def test_host_nearest_edge_cases(ax):
    p = uniform_points(10, 143)
    q = uniform_points(300, 144)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    # k above the tree size, no distances, unsorted predicates
    oh = torch.empty(301, dtype=torch.int32)
    ih = torch.empty(300 * 10, dtype=torch.int32)
    ax.query_nearest_host(bvh, torch.from_numpy(q), 25, oh, ih, chunk=64,
                          policy=ax.TraversalPolicy(0, False))
    ind, off = ax.query(bvh, ax.nearest(cuda(q), 25))
    assert torch.equal(oh, off.cpu()) and torch.equal(ih, ind.cpu())
    # k = 0 and no queries
    oh = torch.full((301,), 7, dtype=torch.int32)
    ax.query_nearest_host(bvh, torch.from_numpy(q), 0, oh, torch.empty(0, dtype=torch.int32))
    assert oh.tolist() == [0] * 301
    oh = torch.full((1,), 7, dtype=torch.int32)
    ax.query_nearest_host(bvh, torch.empty((0, 3)), 4, oh, torch.empty(0, dtype=torch.int32))
    assert oh.tolist() == [0]
    # an empty tree
    empty = ax.BoundingVolumeHierarchy(cuda(np.zeros((0, 3), np.float32)))
    oh = torch.full((301,), 7, dtype=torch.int32)
    ax.query_nearest_host(empty, torch.from_numpy(q), 3, oh, torch.empty(0, dtype=torch.int32))
    assert oh.tolist() == [0] * 301
    # KDOP trees have no distance
    kd = ax.BoundingVolumeHierarchy(ax.kdop_from(cuda(p), 14), kind=ax.KDOP14)
    with pytest.raises(ax.AbxError):
        ax.query_nearest_host(kd, torch.from_numpy(q), 3, torch.empty(301, dtype=torch.int32),
                              torch.empty(900, dtype=torch.int32))
    assert ax.device_errors() == 0
