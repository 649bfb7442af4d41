"""Pin the CPU oracle to the reference's own known-answer tests.

Every case comes from tests/golden/reference_kats.json (generated from the
reference's Boost.Test sources by tests/golden/make_golden.py) or restates a
reference test's construction (cited per test).  No GPU needed.
"""

import numpy as np
import pytest

from oracle import oracle as o
from tests.helpers import assert_crs_multiset_equal, box_list, manufactured_grid, uniform_points


def test_expand_bits_kats(golden):
    # test/tstDetailsMortonCodes.cpp:22-50
    for case in golden["morton"]["expand_bits32"]:
        assert o.expand_bits32(case["input"], case["n_zero"]) == case["expected"], case
    for case in golden["morton"]["expand_bits64"]:
        assert o.expand_bits64(case["input"], case["n_zero"]) == case["expected"], case


def test_morton_kats(golden):
    # test/tstDetailsMortonCodes.cpp:52-82 (1D, 2D and 3D points)
    for case in golden["morton"]["morton"]:
        f = o.morton32 if case["bits"] == 32 else o.morton64
        assert f(case["point"]) == case["expected"], case


def test_assign_morton_codes(golden):
    # test/tstDetailsTreeConstruction.cpp:33-102: boxes around 7 points
    c = golden["assign_morton_codes"]
    pts = np.asarray(c["points"], np.float32)
    boxes = np.concatenate([pts, pts], axis=1)
    scene = o.scene_bounds(boxes, is_box=True)
    assert scene.tolist() == np.asarray(c["scene"], np.float32).tolist()
    codes = o.morton64_codes(boxes, scene, is_box=True)
    e = lambda v: o.expand_bits64(v, 2)  # noqa: E731
    ref = [4 * e(i) + 2 * e(j) + e(k) for i, j, k in c["anchors"]]
    assert codes.tolist() == ref


def test_indirect_sort():
    # test/tstDetailsTreeConstruction.cpp:119-149
    keys, perm = o.sort_u32([4, 3, 2, 1])
    assert keys.tolist() == [1, 2, 3, 4]
    assert perm.tolist() == [3, 2, 1, 0]
    keys, perm = o.sort_u64([4, 3, 2, 1])
    assert perm.tolist() == [3, 2, 1, 0]


def test_sort_is_stable():
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 7, 1000).astype(np.uint64)
    _, perm = o.sort_u64(keys)
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))


def _dfs_string(leaves, internal, n):
    out = []
    node = n

    def walk(node):
        if node < n:
            out.append("L%d" % node)
            if leaves[node]["rope"] != -1:
                walk(int(leaves[node]["rope"]))
        else:
            out.append("I%d" % (node - n))
            walk(int(internal[node - n]["left_child"]))

    walk(node)
    return "".join(out)


def test_karras_example(golden):
    # test/tstDetailsTreeConstruction.cpp:217-269: exact rope / left-child
    # depth-first order for the 8-key example of Karras
    codes = np.asarray(golden["karras"]["sorted_codes"], np.uint64)
    n = codes.size
    geom = np.zeros((n, 3), np.float32)
    leaves, internal = o.generate_hierarchy(geom, np.arange(n, dtype=np.uint32), codes)
    assert _dfs_string(leaves, internal, n) == golden["karras"]["dfs"]


def _run_case(case):
    leaves = box_list(case["leaves"])
    tree = o.OracleTree(leaves, is_box=True)
    if case["kind"] == "nearest":
        q = np.asarray(case["queries"], np.float32).reshape(-1, 4)
        res = []
        for mode in (o.MODE_ARBORX, o.MODE_ORDERED):
            off, ind, _ = tree.nearest(q[:, :3], q[:, 3].astype(np.int32), mode=mode)
            res.append((off, ind))
        return res
    kind = o.KIND_BOX if case["kind"] == "box" else o.KIND_SPHERE
    q = box_list(case["queries"]) if kind == o.KIND_BOX else np.asarray(case["queries"], np.float32).reshape(-1, 4)
    return [tree.spatial(kind, q)]


def test_degenerate_and_policy_cases(golden):
    # test/tstQueryTreeDegenerate.cpp:25-361, tstQueryTreeTraversalPolicy.cpp
    for case in golden["degenerate"]:
        for off, ind in _run_case(case):
            assert_crs_multiset_equal(off, ind, case["offsets"], case["indices"])


def test_tree_bounds_degenerate():
    # empty tree bounds = default box; single leaf bounds = the leaf
    t = o.OracleTree(np.zeros((0, 6), np.float32), is_box=True)
    assert t.bounds.tolist() == box_list(["empty"])[0].tolist()
    t = o.OracleTree(np.asarray([[0, 0, 0, 1, 1, 1]], np.float32), is_box=True)
    assert t.bounds.tolist() == [0, 0, 0, 1, 1, 1]


def test_manufactured_grid():
    # test/tstQueryTreeManufacturedSolution.cpp:29-270
    leaves, cases = manufactured_grid()
    tree = o.OracleTree(leaves, is_box=True)
    for q, (eoff, eind) in cases:
        off, ind = tree.spatial(o.KIND_BOX, q)
        assert_crs_multiset_equal(off, ind, eoff, eind)


def test_stack_capacity():
    # test/tstQueryTreeDegenerate.cpp:367-446: 4096 unit boxes on the
    # diagonal, a query touching all of them, kNN with k = n
    n = 4096
    a = np.arange(n, dtype=np.float32)
    boxes = np.stack([a, a, a, a + 1, a + 1, a + 1], axis=1)
    tree = o.OracleTree(boxes, is_box=True)
    q = box_list(["empty", [0, 0, 0, n, n, n]])
    off, _ = tree.spatial(o.KIND_BOX, q)
    assert off[-1] == n
    for mode in (o.MODE_ARBORX, o.MODE_ORDERED):
        off, ind, _ = tree.nearest(np.zeros((1, 3), np.float32), n, mode=mode)
        assert off[-1] == n and sorted(ind.tolist()) == list(range(n))


@pytest.mark.parametrize("n,nq,k", [(1000, 300, 1), (5000, 500, 10), (20000, 300, 16), (3, 10, 5)])
def test_oracle_knn_matches_brute_force(n, nq, k):
    p = uniform_points(n, 1)
    q = uniform_points(nq, 2)
    tree = o.OracleTree(p)
    off, ind, dist = tree.nearest(q, k)
    bi, bd = o.knn_brute(p, q, k)
    kk = min(k, n)
    assert np.array_equal(off, np.arange(nq + 1) * kk)
    assert np.array_equal(ind.reshape(nq, kk), bi)
    assert np.array_equal(dist.reshape(nq, kk), bd)
    # verbatim ArborX rule: same distances, sets equal up to ties at the k-th
    off2, ind2, dist2 = tree.nearest(q, k, mode=o.MODE_ARBORX)
    assert np.array_equal(np.sort(dist2.reshape(nq, kk), axis=1), bd)


def test_oracle_knn_fp64_check():
    # every float32 distance is the correctly rounded chain of the formula;
    # against float64 it is within a few ulps
    p = uniform_points(4000, 3)
    q = uniform_points(200, 4)
    tree = o.OracleTree(p)
    off, ind, dist = tree.nearest(q, 8)
    d64 = np.sqrt(((p[ind].astype(np.float64) - np.repeat(q, 8, axis=0).astype(np.float64)) ** 2).sum(1))
    assert np.all(np.abs(dist - d64) <= 4 * np.spacing(dist.astype(np.float32)).astype(np.float64) + 1e-12)


@pytest.mark.parametrize("kind", [o.KIND_SPHERE, o.KIND_BOX])
def test_oracle_spatial_matches_brute_force(kind):
    p = uniform_points(20000, 5)
    c = uniform_points(500, 6)
    if kind == o.KIND_SPHERE:
        preds = np.concatenate([c, np.full((500, 1), 0.05, np.float32)], axis=1)
    else:
        preds = np.concatenate([c - 0.04, c + 0.04], axis=1).astype(np.float32)
    tree = o.OracleTree(p)
    off, ind = tree.spatial(kind, preds)
    boff, bind = o.spatial_brute(p, kind, preds)
    assert_crs_multiset_equal(off, ind, boff, bind)


def test_oracle_duplicates_and_line():
    # adversarial inputs: all-equal points and points on a line
    same = np.ones((257, 3), np.float32)
    line = np.repeat(np.linspace(0, 1, 300, dtype=np.float32)[:, None], 3, axis=1)
    for p in (same, line):
        tree = o.OracleTree(p)
        q = uniform_points(50, 7)
        off, ind, dist = tree.nearest(q, 7)
        bi, bd = o.knn_brute(p, q, 7)
        assert np.array_equal(ind.reshape(-1, 7), bi)
        assert np.array_equal(dist.reshape(-1, 7), bd)


def test_oracle_neighbor_lists_golden(golden):
    """test/tstNeighborList.cpp:136-171: full neighbor lists of four points on
    the diagonal (rows compared as multisets, as the reference does)."""
    nl = golden["neighbor_lists"]
    pts = np.asarray(nl["points"], np.float32)
    for case in nl["cases"]:
        sph = np.concatenate([pts, np.full((4, 1), case["radius"], np.float32)], axis=1)
        off, ind = o.spatial_brute(pts, o.KIND_SPHERE, sph)
        rows = [sorted(int(v) for v in ind[off[i]:off[i + 1]] if v != i) for i in range(4)]
        want = [sorted(case["indices"][case["offsets"][i]:case["offsets"][i + 1]]) for i in range(4)]
        assert rows == want


def test_oracle_rays_golden(golden):
    """test/tstRay.cpp:17-275: ray-box intersects / intersection (tolerance
    1e-6 as the test) / distance against the unit box, rays normalized as the
    Ray constructor does."""
    g = golden["rays"]
    box = np.asarray(g["unit_box"], np.float32)
    for c in g["intersects_box"]:
        ray = o.ray_normalize(np.asarray(c["ray"], np.float32))[0]
        assert o.ray_box_intersects(ray, box) == c["hit"], c
    for c in g["intersection"]:
        ray = o.ray_normalize(np.asarray(c["ray"], np.float32))[0]
        hit, t0, t1 = o.ray_box_intersection(ray, box)
        if "hit" in c and not c["hit"]:
            assert not hit and (t0 == np.inf or t1 == -np.inf), c
        else:
            assert hit, c
            assert t0 == pytest.approx(c["t0"], rel=1e-6, abs=1e-30), c
            assert t1 == pytest.approx(c["t1"], rel=1e-6, abs=1e-30), c
    for c in g["distance"]:
        ray = o.ray_normalize(np.asarray(c["ray"], np.float32))[0]
        want = np.inf if c["distance"] == "inf" else c["distance"]
        assert o.ray_box_distance(ray, box) == want


def test_oracle_ray_tree_cases_golden(golden):
    """test/tstQueryTreeRay.cpp:62-265 through the brute-force restatement."""
    g = golden["rays"]
    boxes = np.asarray(g["tree_boxes"], np.float32)
    r = o.ray_normalize(np.asarray([g["tree_intersects"]["ray"]], np.float32))
    off, ind, _ = o.ray_brute(boxes, r, ordered=False)
    assert ind.tolist() == g["tree_intersects"]["indices"]
    for c in g["tree_ordered"]:
        off, ind, _ = o.ray_brute(boxes, o.ray_normalize(np.asarray([c["ray"]], np.float32)), ordered=True)
        assert ind.tolist() == c["indices"]
    one = g["single_leaf"]
    off, ind, _ = o.ray_brute(np.asarray([one["box"]], np.float32),
                              o.ray_normalize(np.asarray(one["rays"], np.float32)), ordered=True)
    assert off.tolist() == one["offsets"] and ind.tolist() == one["indices"]


@pytest.mark.parametrize("k", [6, 14, 18, 26])
def test_oracle_kdop_geometry_golden(golden, k):
    """test/tstGeometryIntersects.cpp:384-571: KDOP-KDOP and KDOP-box against
    empty operands, and the per-k answers of points against a unit cube with
    an edge or a corner cut off."""
    g = golden["kdops"]
    nd = o.KDOP_NDIR[k]
    x = o.kdop_empty(nd)
    assert o.kdop_intersects(x, x) == g["kdop_kdop"]["self_before"]
    unit = np.asarray(g["kdop_box"]["unit_box"], np.float32)
    empty_box = np.array([np.finfo(np.float32).max] * 3 + [-np.finfo(np.float32).max] * 3, np.float32)
    assert o.kdop_intersects(x, empty_box) == g["kdop_box"]["before"]["empty"]
    assert o.kdop_intersects(x, unit) == g["kdop_box"]["before"]["unit"]
    for p in g["kdop_kdop"]["expand"]:
        o.kdop_expand(x, p)
    assert o.kdop_intersects(x, x) == g["kdop_kdop"]["self_after"]
    assert o.kdop_intersects(x, o.kdop_empty(nd)) == g["kdop_kdop"]["empty_after"]
    assert o.kdop_intersects(x, empty_box) == g["kdop_box"]["after"]["empty"]
    assert o.kdop_intersects(x, unit) == g["kdop_box"]["after"]["unit"]
    for poly in g["point_kdop"]:
        x = o.kdop_empty(nd)
        for p in poly["expand"]:
            o.kdop_expand(x, p)
        for c in poly["checks"]:
            assert o.kdop_intersects(x, c["point"]) == c["expected"][str(k)], (k, c)


def test_oracle_kdop_query_golden(golden):
    """test/tstQueryTreeIntersectsKDOP.cpp:26-91: intersects(KDOP<3, 18>) over
    13 points finds {1, 4, 7, 8}; no predicates give offsets {0}."""
    t = golden["kdops"]["tree"]
    x = o.kdop_empty(9)
    for p in t["kdop18_expand"]:
        o.kdop_expand(x, p)
    pts = np.asarray(t["points"], np.float32)
    off, ind = o.kdop_spatial_brute(pts, "point", x[None], 18)
    assert off.tolist() == t["query"]["offsets"] and sorted(ind.tolist()) == t["query"]["indices"]
    off, ind = o.kdop_spatial_brute(pts, "point", np.zeros((0, 18), np.float32), 18)
    assert off.tolist() == t["empty"]["offsets"] and ind.tolist() == t["empty"]["indices"]


def test_oracle_kdop_conversions():
    """A point's KDOP has zero-width ranges at its projections; a box's KDOP
    holds each of its corners and the box's own ranges on the axes; the axis
    boxes of those KDOPs give the boxes back (expand(Box, KDOP))."""
    rng = np.random.default_rng(5)
    lo = rng.random((200, 3), dtype=np.float32)
    boxes = np.concatenate([lo, lo + rng.random((200, 3), dtype=np.float32)], axis=1)
    for k, nd in o.KDOP_NDIR.items():
        kb = o.kdop_from_geometry(boxes, nd, is_box=True)
        assert np.array_equal(o.kdop_axis_boxes(kb), boxes)
        kp = o.kdop_from_geometry(lo, nd)
        assert np.array_equal(kp[:, :nd], kp[:, nd:])
        assert np.array_equal(kp[:, :3], lo)
        for i in range(0, 200, 37):
            for c in range(8):
                corner = [boxes[i, 3 * ((c >> 2) & 1)], boxes[i, 1 + 3 * (c & 1)], boxes[i, 2 + 3 * ((c >> 1) & 1)]]
                assert o.kdop_intersects(kb[i], corner)
    # an inverted box leaves the KDOP empty (ArborX_Expand.hpp:163-165)
    bad = np.array([[1, 0, 0, 0, 1, 1]], np.float32)
    assert np.array_equal(o.kdop_from_geometry(bad, 7, is_box=True)[0], o.kdop_empty(7))


def _golden_geometry(g):
    kind, v = g
    if kind == "box" and v == "empty":
        return "box", np.array([[np.float32(3.40282347e38)] * 3 + [np.float32(-3.40282347e38)] * 3],
                               np.float32)
    return kind, np.asarray([v], np.float32)


def test_oracle_geometry_golden(golden):
    """test/tstGeometryIntersects.cpp:44-126 and test/tstGeometryDistance.cpp:
    39-67 through the oracle's brute force (one value, one predicate; a point
    predicate is the degenerate box [p, p])."""
    g = golden["geometry"]
    for c in g["intersects"]:
        got = []
        for a, b in ((c["a"], c["b"]), (c["b"], c["a"])):
            vk, vals = _golden_geometry(a)
            pk, pred = _golden_geometry(b)
            if vk == "sphere":
                continue  # values are points or boxes
            if pk == "point":
                pk, pred = "box", np.concatenate([pred, pred], axis=1)
            kind = o.KIND_SPHERE if pk == "sphere" else o.KIND_BOX
            off, _ = o.spatial_brute(vals, kind, pred, is_box=vk == "box")
            got.append(bool(off[-1]))
        assert got and all(x == c["expected"] for x in got), c
    for c in g["distance"]:
        _, q = _golden_geometry(c["a"])
        bk, vals = _golden_geometry(c["b"])
        _, d = o.knn_brute(vals, q, 1, is_box=bk == "box")
        e = c["expected"]
        want = np.sqrt(np.float32(e["sqrt_of"])) if "sqrt_of" in e else np.float32(e["value"])
        assert d[0, 0] == want, c


def test_oracle_expand_half_to_full_golden(golden):
    """test/tstDetailsExpandHalfToFull.cpp:48-80 (rows compared as multisets,
    as the reference does)."""
    for c in golden["expand_half_to_full"]["cases"]:
        off, ind = o.expand_half_to_full(c["offsets_in"], c["indices_in"])
        assert off == c["offsets_out"]
        rows = [sorted(ind[off[i]:off[i + 1]]) for i in range(len(off) - 1)]
        want = [sorted(c["indices_out"][off[i]:off[i + 1]]) for i in range(len(off) - 1)]
        assert rows == want
