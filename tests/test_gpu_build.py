"""GPU parity of the construction path against the CPU oracle: scene bounds,
Morton codes, the stable radix sort, the hierarchy, and whole trees.  Every
comparison is bit-exact (integers and float32 bit patterns)."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.int32)


def test_scene_bounds_points_and_boxes(ax):
    for n in (1, 3, 4, 5, 1000, 1 << 20 | 3):
        p = uniform_points(n, n) * 7 - 3
        got = ax.scene_bounds(cuda(p)).cpu().numpy()
        assert np.array_equal(bits(got), bits(o.scene_bounds(p)))
    b = np.concatenate([uniform_points(5000, 1), uniform_points(5000, 2) + 1], axis=1)
    got = ax.scene_bounds(cuda(b), kind=1).cpu().numpy()
    assert np.array_equal(bits(got), bits(o.scene_bounds(b, is_box=True)))


def test_assign_morton_codes_golden(ax, golden):
    # test/tstDetailsTreeConstruction.cpp:33-102
    c = golden["assign_morton_codes"]
    pts = np.asarray(c["points"], np.float32)
    boxes = np.concatenate([pts, pts], axis=1)
    scene = ax.scene_bounds(cuda(boxes), kind=1)
    assert scene.cpu().numpy().tolist() == np.asarray(c["scene"], np.float32).tolist()
    codes = ax.morton64(cuda(boxes), scene, kind=1).cpu().numpy().view(np.uint64)
    e = lambda v: o.expand_bits64(v, 2)  # noqa: E731
    assert codes.tolist() == [4 * e(i) + 2 * e(j) + e(k) for i, j, k in c["anchors"]]


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_morton_codes_match_oracle(ax, kind):
    rng = np.random.default_rng(11 + kind)
    n = 100003
    cols = {0: 3, 1: 6, 2: 4}[kind]
    g = (rng.random((n, cols), dtype=np.float32) * 3 - 1).astype(np.float32)
    if kind == 1:
        g[:, 3:] = g[:, :3] + np.abs(g[:, 3:]) * 0.1
    scene = np.asarray([0, 0, 0, 1, 1, 1], np.float32)  # points outside clamp
    got64 = ax.morton64(cuda(g), cuda(scene), kind=kind).cpu().numpy().view(np.uint64)
    if kind != 2:
        ref64 = o.morton64_codes(g, scene, is_box=(kind == 1))
        assert np.array_equal(got64, ref64)
    got32 = ax.morton32(cuda(g), cuda(scene), kind=kind).cpu().numpy().view(np.uint32)
    okind = {0: o.KIND_POINT, 1: o.KIND_BOX, 2: o.KIND_SPHERE}[kind]
    assert np.array_equal(got32, o.morton32_codes(g, scene, okind))


@pytest.mark.parametrize("n", [1, 2, 5, 4095, 4096, 4097, 100000, 3 * 4096 * 7 + 11, 1 << 21])
def test_sort_u64_stable(ax, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    keys[1::2] = keys[0::2][: len(keys[1::2])]  # duplicates
    keys[: n // 4] &= np.uint64(0xFF00FF)  # many equal low digits
    t = cuda(keys.view(np.int64))
    perm = ax.sort_u64(t).cpu().numpy().view(np.uint32)
    sk, sp = o.sort_u64(keys)
    assert np.array_equal(t.cpu().numpy().view(np.uint64), sk)
    assert np.array_equal(perm, sp)


@pytest.mark.parametrize("n", [1, 3, 4096, 65537, 1000003])
def test_sort_u32_stable(ax, n):
    rng = np.random.default_rng(n + 1)
    keys = rng.integers(0, 1 << 30, size=n, dtype=np.uint32)
    keys[n // 2:] = keys[n // 2:] % 17
    t = cuda(keys.view(np.int32))
    perm = ax.sort_u32(t).cpu().numpy().view(np.uint32)
    sk, sp = o.sort_u32(keys)
    assert np.array_equal(t.cpu().numpy().view(np.uint32), sk)
    assert np.array_equal(perm, sp)


def test_indirect_sort_golden(ax):
    # test/tstDetailsTreeConstruction.cpp:119-149
    t = cuda(np.asarray([4, 3, 2, 1], np.int32))
    perm = ax.sort_u32(t).cpu().numpy()
    assert t.cpu().numpy().tolist() == [1, 2, 3, 4]
    assert perm.tolist() == [3, 2, 1, 0]


def test_karras_example(ax, golden):
    # test/tstDetailsTreeConstruction.cpp:217-269
    from tests.test_oracle_golden import _dfs_string

    codes = np.asarray(golden["karras"]["sorted_codes"], np.uint64)
    n = codes.size
    geom = np.zeros((n, 3), np.float32)
    leaves, internal = ax.generate_hierarchy(
        cuda(geom), cuda(np.arange(n, dtype=np.int32)), cuda(codes.view(np.int64))
    )
    lv = np.zeros(n, o.LEAF_DTYPE)
    lv["rope"], lv["value"] = leaves.cpu().numpy()[:, 0], leaves.cpu().numpy()[:, 1]
    it = internal.cpu().numpy().view(o.INTERNAL_DTYPE).reshape(-1)
    assert _dfs_string(lv, it, n) == golden["karras"]["dfs"]


def _tree_arrays_equal(bvh, ref):
    leaves, internal = bvh.export_nodes()
    leaves = leaves.cpu().numpy()
    assert np.array_equal(leaves[:, 0], ref.leaves["rope"])
    assert np.array_equal(leaves[:, 1], ref.leaves["value"])
    got = internal.cpu().numpy()
    want = ref.internal.view(np.int32).reshape(-1, 8)
    assert np.array_equal(got, want)
    assert np.array_equal(bits(np.asarray(bvh.bounds(), np.float32)), bits(ref.bounds))


@pytest.mark.parametrize("n", [2, 3, 7, 100, 10007, 500000])
def test_tree_arrays_bit_exact_points(ax, n):
    p = uniform_points(n, 100 + n)
    bvh = ax.BoundingVolumeHierarchy(cuda(p))
    _tree_arrays_equal(bvh, o.OracleTree(p))


def test_tree_arrays_bit_exact_duplicates_and_lines(ax):
    same = np.ones((1000, 3), np.float32)
    line = np.repeat(np.linspace(0, 1, 4099, dtype=np.float32)[:, None], 3, axis=1)
    mixed = np.concatenate([uniform_points(3000, 9), same[:500], uniform_points(3000, 9)[:700]])
    for p in (same, line, mixed):
        bvh = ax.BoundingVolumeHierarchy(cuda(p))
        _tree_arrays_equal(bvh, o.OracleTree(p))


def test_tree_arrays_bit_exact_boxes(ax):
    lo = uniform_points(20000, 21) * 10
    hi = lo + uniform_points(20000, 22)
    b = np.concatenate([lo, hi], axis=1)
    bvh = ax.BoundingVolumeHierarchy(cuda(b), kind=1)
    _tree_arrays_equal(bvh, o.OracleTree(b, is_box=True))


def test_empty_and_single_leaf_trees(ax):
    empty = ax.BoundingVolumeHierarchy(torch.zeros((0, 6), device="cuda"), kind=1)
    assert empty.empty() and empty.size() == 0
    f = np.finfo(np.float32).max
    assert empty.bounds() == (f, f, f, -f, -f, -f)
    one = ax.BoundingVolumeHierarchy(cuda(np.asarray([[0, 0, 0, 1, 1, 1]], np.float32)), kind=1)
    assert one.size() == 1 and one.bounds() == (0, 0, 0, 1, 1, 1)
    leaves, internal = one.export_nodes()
    assert leaves.cpu().numpy().tolist() == [[-1, 0]] and internal.numel() == 0


def test_build_is_deterministic(ax):
    p = uniform_points(300000, 5)
    t = cuda(p)
    first = [x.cpu().numpy() for x in ax.BoundingVolumeHierarchy(t).export_nodes()]
    for _ in range(3):
        again = [x.cpu().numpy() for x in ax.BoundingVolumeHierarchy(t).export_nodes()]
        assert all(np.array_equal(a, b) for a, b in zip(first, again))
    assert ax.device_errors() == 0


def _hybrid_cases(n, seed):
    rng = np.random.default_rng(seed)
    uniform = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    # clustered: few distinct top digits, random low bits (long runs)
    clustered = (rng.integers(0, 50, n, dtype=np.uint64) << np.uint64(40)) | rng.integers(
        0, 1 << 20, n, dtype=np.uint64)
    same_top = np.uint64(7 << 50) | rng.integers(0, 8, n, dtype=np.uint64)
    equal = np.full(n, 12345, np.uint64)
    mixed = uniform.copy()
    mixed[: n // 3] = clustered[: n // 3]
    return [uniform, clustered, same_top, equal, mixed]


@pytest.mark.parametrize("top", ["0", "3", "4"])
def test_sort_u64_hybrid_top_passes(ax, top):
    """The top-digit passes + run fix-up (+ long-run segmented sort) give the
    full stable sort on uniform, clustered, one-run and all-equal keys."""
    from arborx_gb300 import _lib

    L = _lib.load()
    L.abx_tuning_set(b"SORT_TOP_PASSES", int(top))
    try:
        for keys in _hybrid_cases(300007, 5):
            t = cuda(keys.view(np.int64))
            perm = ax.sort_u64(t).cpu().numpy().view(np.uint32)
            ref = np.argsort(keys, kind="stable")
            assert np.array_equal(perm, ref.astype(np.uint32))
            assert np.array_equal(t.cpu().numpy().view(np.uint64), keys[ref])
    finally:
        L.abx_tuning_reset()
    assert ax.device_errors() == 0


def test_sort_u32_hybrid(ax):
    rng = np.random.default_rng(6)
    n = 500009
    for keys in (rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32),
                 (rng.integers(0, 3, n, dtype=np.uint32) << np.uint32(8)) | rng.integers(0, 256, n, dtype=np.uint32)):
        t = cuda(keys.view(np.int32))
        perm = ax.sort_u32(t).cpu().numpy().view(np.uint32)
        ref = np.argsort(keys, kind="stable").astype(np.uint32)
        assert np.array_equal(perm, ref)
        assert np.array_equal(t.cpu().numpy().view(np.uint32), keys[ref])


def test_strided_values_build_the_same_tree(ax):
    """Access traits: column-major (SoA), padded float4 and sliced views build
    exactly the tree of the row-major copy (ArborX_AccessTraits.hpp:36-76)."""
    p = uniform_points(50000, 77)
    ref = [x.cpu().numpy() for x in ax.BoundingVolumeHierarchy(cuda(p)).export_nodes()]
    soa = cuda(np.ascontiguousarray(p.T)).t()            # strides (1, n)
    pad = cuda(np.concatenate([p, np.zeros((p.shape[0], 1), np.float32)], axis=1))[:, :3]  # (4, 1)
    big = cuda(np.repeat(p, 2, axis=0))[::2]             # (6, 1)
    for v in (soa, pad, big):
        assert not v.is_contiguous()
        got = [x.cpu().numpy() for x in ax.BoundingVolumeHierarchy(v).export_nodes()]
        assert all(np.array_equal(a, b) for a, b in zip(ref, got))
    lo = uniform_points(3000, 78)
    b = np.concatenate([lo, lo + 0.01], axis=1)
    refb = [x.cpu().numpy() for x in ax.BoundingVolumeHierarchy(cuda(b), kind=1).export_nodes()]
    bsoa = cuda(np.ascontiguousarray(b.T)).t()
    gotb = [x.cpu().numpy() for x in ax.BoundingVolumeHierarchy(bsoa, kind=1).export_nodes()]
    assert all(np.array_equal(x, y) for x, y in zip(refb, gotb))
