"""A nearest query captured in a CUDA graph (abx_bvh_query_nearest_into):
replays give the results of the direct query, also after the query points
were overwritten in place."""

import numpy as np
import pytest
import torch

from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _direct(ax, bvh, q, k):
    i, o, d = ax.query(bvh, ax.nearest(q, k), with_distances=True)
    return i.cpu().numpy(), o.cpu().numpy(), d.cpu().numpy()


@pytest.mark.parametrize("k", [16, 40])
def test_captured_nearest_replays_match_direct_queries(ax, k):
    bvh = ax.BoundingVolumeHierarchy(cuda(uniform_points(200000, 90)))
    bvh.bounds()  # the build has completed before capture
    nq = 100003
    q = cuda(uniform_points(nq, 91))
    off = torch.empty(nq + 1, dtype=torch.int32, device="cuda")
    idx = torch.empty(nq * k, dtype=torch.int32, device="cuda")
    dist = torch.empty(nq * k, dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ax.query_nearest_into(bvh, q, k, off, idx, dist, space=s)  # warm-up, not captured
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ax.query_nearest_into(bvh, q, k, off, idx, dist, space=s)
    for seed in (92, 93):
        q.copy_(cuda(uniform_points(nq, seed)))
        idx.zero_()
        dist.zero_()
        g.replay()
        torch.cuda.synchronize()
        ri, ro, rd = _direct(ax, bvh, q, k)
        assert np.array_equal(off.cpu().numpy(), ro)
        assert np.array_equal(idx.cpu().numpy(), ri)
        assert np.array_equal(dist.cpu().numpy().view(np.int32), rd.view(np.int32))
    assert ax.device_errors() == 0


def test_nearest_into_without_capture_and_edge_cases(ax):
    bvh = ax.BoundingVolumeHierarchy(cuda(uniform_points(1000, 94)))
    q = cuda(uniform_points(77, 95))
    off = torch.empty(78, dtype=torch.int32, device="cuda")
    idx = torch.empty(77 * 5, dtype=torch.int32, device="cuda")
    ax.query_nearest_into(bvh, q, 5, off, idx)
    ri, ro, _ = _direct(ax, bvh, q, 5)
    assert np.array_equal(off.cpu().numpy(), ro) and np.array_equal(idx.cpu().numpy(), ri)
    ax.query_nearest_into(bvh, q, 0, off, idx)
    assert off.cpu().numpy().tolist() == [0] * 78
