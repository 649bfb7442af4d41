"""GPU parity of the query path (spatial and nearest, CRS output) against the
CPU oracle and the reference's known-answer cases.

Spatial results are compared exactly, order included: the GPU depth-first
walk visits leaves in the reference's rope order.  Nearest results are the k
smallest (distance, index) pairs in ascending order: indices and float32
distances must be bit-identical to the oracle."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import assert_crs_multiset_equal, box_list, manufactured_grid, uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


POLICIES = [(0, True), (0, False), (40, True), (-64, True), (3, True)]


def _spheres(centres, r):
    return np.concatenate([centres, np.full((len(centres), 1), r, np.float32)], axis=1).astype(np.float32)


def _run_golden_case(ax, case, policy):
    leaves = box_list(case["leaves"])
    bvh = ax.BoundingVolumeHierarchy(cuda(leaves), kind=1)
    if case["kind"] == "nearest":
        q = np.asarray(case["queries"], np.float32).reshape(-1, 4)
        k = cuda(q[:, 3].astype(np.int32))
        preds = ax.nearest(cuda(np.ascontiguousarray(q[:, :3])), k)
    elif case["kind"] == "box":
        preds = ax.intersects(cuda(box_list(case["queries"])))
    else:
        preds = ax.intersects(cuda(np.asarray(case["queries"], np.float32).reshape(-1, 4)))
    ind, off = ax.query(bvh, preds, policy)
    return host(off), host(ind)


def test_golden_degenerate_cases(ax, golden):
    # test/tstQueryTreeDegenerate.cpp:25-361, tstQueryTreeTraversalPolicy.cpp
    for case in golden["degenerate"]:
        for b, s in POLICIES:
            if case["kind"] == "nearest" and b != 0:
                continue
            off, ind = _run_golden_case(ax, case, ax.TraversalPolicy(b if b >= 0 else 0, s))
            assert_crs_multiset_equal(off, ind, case["offsets"], case["indices"])


def test_golden_buffer_policy(ax, golden):
    # test/tstQueryTreeTraversalPolicy.cpp:32-130
    case = [c for c in golden["degenerate"] if "buffer_sizes_ok" in c][0]
    for b in case["buffer_sizes_ok"]:
        off, ind = _run_golden_case(ax, case, ax.TraversalPolicy().setBufferSize(b))
        assert_crs_multiset_equal(off, ind, case["offsets"], case["indices"])
    for b in case["buffer_sizes_throw"]:
        with pytest.raises(ax.SearchException):
            _run_golden_case(ax, case, ax.TraversalPolicy().setBufferSize(b))


def test_manufactured_grid(ax):
    # test/tstQueryTreeManufacturedSolution.cpp:29-270
    leaves, cases = manufactured_grid()
    bvh = ax.BoundingVolumeHierarchy(cuda(leaves), kind=1)
    for q, (eoff, eind) in cases:
        for b, s in POLICIES:
            ind, off = ax.query(bvh, ax.intersects(cuda(q)), ax.TraversalPolicy(b, s))
            assert_crs_multiset_equal(host(off), host(ind), eoff, eind)


def test_stack_capacity(ax):
    # test/tstQueryTreeDegenerate.cpp:367-446
    n = 4096
    a = np.arange(n, dtype=np.float32)
    boxes = np.stack([a, a, a, a + 1, a + 1, a + 1], axis=1)
    bvh = ax.BoundingVolumeHierarchy(cuda(boxes), kind=1)
    ind, off = ax.query(bvh, ax.intersects(cuda(box_list(["empty", [0, 0, 0, n, n, n]]))))
    assert host(off).tolist() == [0, 0, n]
    ind, off = ax.query(bvh, ax.nearest(cuda(np.zeros((1, 3), np.float32)), n))
    assert host(off).tolist() == [0, n] and sorted(host(ind).tolist()) == list(range(n))
    assert ax.device_errors() == 0


@pytest.mark.parametrize("kind", ["sphere", "box"])
@pytest.mark.parametrize("n,nq", [(2, 50), (1000, 2000), (200000, 20000)])
def test_spatial_matches_oracle_exactly(ax, kind, n, nq):
    p = uniform_points(n, 31 + n)
    c = uniform_points(nq, 37 + nq)
    r = np.float32((32 * 3 / (4 * np.pi * n)) ** (1 / 3))
    if kind == "sphere":
        preds = _spheres(c, r)
        okind = o.KIND_SPHERE
    else:
        preds = np.concatenate([c - r, c + r], axis=1).astype(np.float32)
        okind = o.KIND_BOX
    ref = o.OracleTree(p)
    roff, rind = ref.spatial(okind, preds)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    for b, s in POLICIES:
        ind, off = ax.query(bvh, ax.intersects(cuda(preds)), ax.TraversalPolicy(b if b >= 0 else 128, s))
        assert np.array_equal(host(off), roff)
        assert np.array_equal(host(ind), rind)  # same order as the rope walk


def test_spatial_on_box_tree(ax):
    lo = uniform_points(30000, 41) * 10
    b = np.concatenate([lo, lo + uniform_points(30000, 42) * 0.3], axis=1)
    q = uniform_points(3000, 43) * 10
    spheres = _spheres(q, 0.25)
    boxes = np.concatenate([q - 0.2, q + 0.2], axis=1).astype(np.float32)
    ref = o.OracleTree(b, is_box=True)
    bvh = ax.BoundingVolumeHierarchy(cuda(b), kind=1)
    for preds, okind in ((spheres, o.KIND_SPHERE), (boxes, o.KIND_BOX)):
        roff, rind = ref.spatial(okind, preds)
        ind, off = ax.query(bvh, ax.intersects(cuda(preds)))
        assert np.array_equal(host(off), roff) and np.array_equal(host(ind), rind)


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 10, 16, 17, 32, 33, 100])
def test_nearest_matches_oracle_bit_exact(ax, k):
    n, nq = 50000, 4000
    p = uniform_points(n, 51)
    q = uniform_points(nq, 52)
    ref = o.OracleTree(p)
    roff, rind, rdist = ref.nearest(q, k)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    for s in (True, False):
        ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), k), ax.TraversalPolicy(0, s), with_distances=True)
        assert np.array_equal(host(off), roff)
        assert np.array_equal(host(ind), rind)
        assert np.array_equal(host(dist).view(np.int32), rdist.view(np.int32))
        ind2, off2 = ax.query(bvh, ax.nearest(cuda(q), k), ax.TraversalPolicy(0, s))
        assert np.array_equal(host(ind2), rind)


def test_nearest_matches_brute_force_and_fp64(ax):
    n, nq, k = 20000, 1000, 16
    p = uniform_points(n, 61)
    q = uniform_points(nq, 62)
    bi, bd = o.knn_brute(p, q, k)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), k), with_distances=True)
    assert np.array_equal(host(ind).reshape(nq, k), bi)
    assert np.array_equal(host(dist).reshape(nq, k), bd)
    d64 = np.sqrt(((p[bi.reshape(-1)].astype(np.float64) - np.repeat(q, k, 0).astype(np.float64)) ** 2).sum(1))
    assert np.all(np.abs(host(dist) - d64) <= 4 * np.spacing(host(dist)))


def test_nearest_ties_broken_by_index(ax):
    # every query is equidistant from many duplicated points
    p = np.concatenate([np.ones((100, 3), np.float32), np.zeros((100, 3), np.float32)])
    q = np.full((10, 3), 0.5, np.float32)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), 7), with_distances=True)
    assert host(ind).reshape(10, 7).tolist() == [list(range(7))] * 10
    bi, _ = o.knn_brute(p, q, 7)
    assert np.array_equal(host(ind).reshape(10, 7), bi)


def test_nearest_per_query_k_and_underflow(ax):
    n = 30
    p = uniform_points(n, 71)
    q = uniform_points(500, 72)
    k = np.random.default_rng(73).integers(-2, 70, size=500).astype(np.int32)
    ref = o.OracleTree(p)
    roff, rind, rdist = ref.nearest(q, k)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), cuda(k)), with_distances=True)
    assert np.array_equal(host(off), roff)
    assert np.array_equal(host(ind), rind)
    assert np.array_equal(host(dist), rdist)
    ind, off = ax.query(bvh, ax.nearest(cuda(q), 50))  # k > n for every query
    roff, rind, _ = ref.nearest(q, 50)
    assert np.array_equal(host(off), roff) and np.array_equal(host(ind), rind)


def test_nearest_on_box_tree(ax):
    lo = uniform_points(20000, 81) * 10
    b = np.concatenate([lo, lo + uniform_points(20000, 82)], axis=1)
    q = uniform_points(2000, 83) * 10
    ref = o.OracleTree(b, is_box=True)
    bvh = ax.BoundingVolumeHierarchy(cuda(b), kind=1)
    for k in (1, 8, 40):
        roff, rind, rdist = ref.nearest(q, k)
        ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), k), with_distances=True)
        assert np.array_equal(host(ind), rind) and np.array_equal(host(dist), rdist)


def test_clustered_knn(ax):
    # Gaussian-mixture clouds, with tight clusters (many near-equal codes)
    rng = np.random.default_rng(91)
    centres = rng.random((64, 3))
    sigma = 10 ** rng.uniform(-3, -1, 64)
    comp = rng.integers(0, 64, 200000)
    p = (centres[comp] + rng.normal(size=(200000, 3)) * sigma[comp, None]).astype(np.float32)
    q = (centres[comp[:5000]] + rng.normal(size=(5000, 3)) * sigma[comp[:5000], None]).astype(np.float32)
    ref = o.OracleTree(p)
    roff, rind, rdist = ref.nearest(q, 16)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), 16), with_distances=True)
    assert np.array_equal(host(ind), rind) and np.array_equal(host(dist), rdist)


def test_large_uniform_sampled_parity(ax):
    # full-size tree; a sample of queries is checked against the oracle, and
    # size-independent properties on all of them
    n = 2_000_000
    p = uniform_points(n, 101)
    q = uniform_points(200_000, 102)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), 16), with_distances=True)
    d = host(dist).reshape(-1, 16)
    i = host(ind).reshape(-1, 16)
    assert np.all(np.diff(d, axis=1) >= 0)  # ascending
    assert np.all((i >= 0) & (i < n))
    ref = o.OracleTree(p)
    sample = np.arange(0, 200_000, 97)
    _, rind, rdist = ref.nearest(q[sample], 16)
    assert np.array_equal(i[sample].reshape(-1), rind)
    assert np.array_equal(d[sample].reshape(-1), rdist)
    assert ax.device_errors() == 0


def test_results_do_not_depend_on_predicate_order(ax):
    p = uniform_points(100000, 111)
    q = uniform_points(10000, 112)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    perm = np.random.default_rng(113).permutation(len(q))
    a_ind, a_off = ax.query(bvh, ax.intersects(cuda(_spheres(q, 0.02))))
    b_ind, b_off = ax.query(bvh, ax.intersects(cuda(_spheres(q[perm], 0.02))))
    a = [host(a_ind)[host(a_off)[j]:host(a_off)[j + 1]].tolist() for j in perm]
    b = [host(b_ind)[host(b_off)[j]:host(b_off)[j + 1]].tolist() for j in range(len(q))]
    assert a == b


def test_exclusive_scan_and_crs_query_impl(ax, golden):
    # test/tstDetailsCrsGraphWrapperImpl.cpp:49-101: counts 0..n-1 scan to the
    # reference offsets
    c = golden["crs_query_impl"]
    counts = np.arange(c["n"], dtype=np.int32)
    assert host(ax.exclusive_scan(cuda(counts))).tolist() == c["offsets"]
    big = np.random.default_rng(5).integers(0, 40, size=3_000_001).astype(np.int32)
    got = host(ax.exclusive_scan(cuda(big)))
    assert np.array_equal(got[:-1], o.exclusive_scan(big)) and got[-1] == big.sum()


@pytest.mark.parametrize("bucket", [1, 2, 5, 8, 32])
def test_results_do_not_depend_on_bucket_size(ax, bucket):
    # the query-time bucket limits are tuning knobs: kNN and spatial results
    # (order included) are the same for every value
    L = ax._lib.load()
    p = uniform_points(100000, 121)
    q = uniform_points(20000, 122)
    ref = o.OracleTree(p)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ax._lib.check(L.abx_tuning_set(b"SPATIAL_BUCKET", bucket))
    ax._lib.check(L.abx_tuning_set(b"NEAREST_BUCKET", bucket))
    try:
        _check_variant_results(ax, bvh, ref, q)
    finally:
        L.abx_tuning_reset()


def _check_variant_results(ax, bvh, ref, q):
    for k in (1, 7, 16, 32, 40):
        roff, rind, rdist = ref.nearest(q, k)
        ind, off, dist = ax.query(bvh, ax.nearest(cuda(q), k), with_distances=True)
        assert np.array_equal(host(ind), rind) and np.array_equal(host(dist), rdist)
    spheres = _spheres(q, 0.02)
    roff, rind = ref.spatial(o.KIND_SPHERE, spheres)
    ind, off = ax.query(bvh, ax.intersects(cuda(spheres)))
    assert np.array_equal(host(off), roff) and np.array_equal(host(ind), rind)
    boxes = np.concatenate([q - 0.01, q + 0.01], axis=1).astype(np.float32)
    roff, rind = ref.spatial(o.KIND_BOX, boxes)
    ind, off = ax.query(bvh, ax.intersects(cuda(boxes)))
    assert np.array_equal(host(off), roff) and np.array_equal(host(ind), rind)
    assert ax.device_errors() == 0



def test_one_pass_spatial_equals_two_pass(ax):
    # default policy: from 65536 queries on, a sampled buffer takes the
    # counting pass's results and only overflowing queries are traversed
    # again; the CRS (order included) equals the plain two-pass result
    L = ax._lib.load()
    p = uniform_points(300000, 141)
    q = uniform_points(150000, 142)
    rng = np.random.default_rng(7)
    r = np.where(rng.random(q.shape[0]) < 0.02, 0.08, 0.012).astype(np.float32)  # 2% heavy
    spheres = np.concatenate([q, r[:, None]], axis=1)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    ref = o.OracleTree(p)
    roff, rind = ref.spatial(o.KIND_SPHERE, spheres)
    try:
        for one_pass in (0, 1):
            ax._lib.check(L.abx_tuning_set(b"SPATIAL_ONE_PASS", one_pass))
            for sort in (True, False):
                pol = ax.TraversalPolicy().setPredicateSorting(sort)
                ind, off = ax.query(bvh, ax.intersects(cuda(spheres)), pol)
                assert np.array_equal(host(off), roff) and np.array_equal(host(ind), rind)
        # an explicit small buffer overflows for the heavy queries only
        ind, off = ax.query(bvh, ax.intersects(cuda(spheres)), ax.TraversalPolicy().setBufferSize(8))
        assert np.array_equal(host(off), roff) and np.array_equal(host(ind), rind)
    finally:
        L.abx_tuning_reset()
    assert ax.device_errors() == 0
