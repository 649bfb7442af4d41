"""Generate tests/golden/reference_kats.json from the reference's test files.

Run in a container that has the ArborX sources mounted:

    python tests/golden/make_golden.py /root/reference

The known-answer vectors are read out of the reference's Boost.Test sources as
text (regular expressions over the assertion lines), so the fixture follows
the reference exactly; the structured degenerate / policy cases whose inputs
are spelled as C++ initialiser lists are transcribed below with the file:line
they come from.  The JSON is committed; tests never read the reference tree.
"""

import json
import os
import re
import sys


def _read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def morton_kats(root):
    """test/tstDetailsMortonCodes.cpp:22-82."""
    src = _read(root, "test/tstDetailsMortonCodes.cpp")
    x32 = int(re.search(r"unsigned x = 0b([01]+)u;", src).group(1), 2)
    y64 = int(re.search(r"unsigned long long y = 0b([01]+)llu;", src).group(1), 2)
    expand32, expand64 = [], []
    for m in re.finditer(r"expandBitsBy<(\d)>\((x|y)\) ==\s+0b([01]+)(u|llu)\);", src):
        n, var, bits = int(m.group(1)), m.group(2), int(m.group(3), 2)
        (expand32 if var == "x" else expand64).append(
            {"n_zero": n, "input": x32 if var == "x" else y64, "expected": bits}
        )
    morton = []
    for m in re.finditer(r"morton(32|64)\(Point\{([^}]*)\}\) == 0x([0-9a-f]+)(u|llu)\);", src):
        coords = [float(c.strip().rstrip("f")) for c in m.group(2).split(",")]
        morton.append({"bits": int(m.group(1)), "point": coords, "expected": int(m.group(3), 16)})
    assert len(expand32) == 10 and len(expand64) == 10 and len(morton) == 22
    return {"expand_bits32": expand32, "expand_bits64": expand64, "morton": morton}


def karras_example(root):
    """test/tstDetailsTreeConstruction.cpp:217-269 (Karras' 8-key example)."""
    src = _read(root, "test/tstDetailsTreeConstruction.cpp")
    block = src[src.index("example_tree_construction"):]
    codes = re.search(r"std::vector<std::string> s\{([^}]*)\}", block).group(1)
    codes = [int(c, 2) for c in re.findall(r'"([01]+)"', codes)]
    ref = re.search(r"ref << ((?:\"[IL]\d\"\s*(?:<<\s*)?)+)", block).group(1)
    dfs = "".join(re.findall(r'"([IL]\d)"', ref))
    assert len(codes) == 8 and len(dfs) == 2 * 15
    return {"sorted_codes": codes, "dfs": dfs}


def assign_morton_codes(root):
    """test/tstDetailsTreeConstruction.cpp:33-102: 7 points, their scene box
    and Morton64 codes 4*e(i) + 2*e(j) + e(k) of the anchor cells."""
    src = _read(root, "test/tstDetailsTreeConstruction.cpp")
    assert "{{1.33, 2.33, 3.33}}" in src and "{{N - 1, N - 1, N - 1}}" in src
    N = 1 << 21
    points = [
        [0.0, 0.0, 0.0],
        [0.25, 0.75, 0.25],
        [0.75, 0.25, 0.25],
        [0.75, 0.75, 0.25],
        [1.33, 2.33, 3.33],
        [1.66, 2.66, 3.66],
        [float(N), float(N), float(N)],
    ]
    anchors = [[0, 0, 0]] * 4 + [[1, 2, 3]] * 2 + [[N - 1, N - 1, N - 1]]
    return {"points": points, "scene": [0.0, 0.0, 0.0, float(N), float(N), float(N)], "anchors": anchors}


def degenerate_cases():
    """test/tstQueryTreeDegenerate.cpp:25-446 and
    test/tstQueryTreeTraversalPolicy.cpp:32-202, transcribed.  Leaves are
    boxes [min xyz, max xyz]; E is the default (empty) box; spheres are
    [cx, cy, cz, r]; nearest queries are [x, y, z, k]."""
    E = "empty"
    unit = [0, 0, 0, 1, 1, 1]
    p0 = [0, 0, 0, 0, 0, 0]
    p1 = [1, 1, 1, 1, 1, 1]
    cases = [
        # empty tree (:25-123)
        {"cite": "tstQueryTreeDegenerate.cpp:57-83", "leaves": [], "kind": "box",
         "queries": [E, E], "indices": [], "offsets": [0, 0, 0]},
        {"cite": "tstQueryTreeDegenerate.cpp:85-101", "leaves": [], "kind": "sphere",
         "queries": [[0, 0, 0, 1], [1, 1, 1, 2]], "indices": [], "offsets": [0, 0, 0]},
        {"cite": "tstQueryTreeDegenerate.cpp:115-122", "leaves": [], "kind": "nearest",
         "queries": [[0, 0, 0, 1], [1, 1, 1, 2]], "indices": [], "offsets": [0, 0, 0]},
        # single leaf (:125-223)
        {"cite": "tstQueryTreeDegenerate.cpp:147-153", "leaves": [unit], "kind": "box",
         "queries": [[5, 5, 5, 5, 5, 5], [.5, .5, .5, .5, .5, .5]], "indices": [0], "offsets": [0, 0, 1]},
        {"cite": "tstQueryTreeDegenerate.cpp:161-168", "leaves": [unit], "kind": "sphere",
         "queries": [[0, 0, 0, 1], [1, 1, 1, 3], [5, 5, 5, 2]], "indices": [0, 0], "offsets": [0, 1, 2, 2]},
        {"cite": "tstQueryTreeDegenerate.cpp:197-200", "leaves": [unit], "kind": "nearest",
         "queries": [[0, 0, 0, 3], [4, 5, 1, 1]], "indices": [0, 0], "offsets": [0, 1, 2]},
        {"cite": "tstQueryTreeDegenerate.cpp:202-209", "leaves": [unit], "kind": "nearest",
         "queries": [[0, 0, 0, 1], [1, 1, 1, 2], [2, 2, 2, 3]], "indices": [0, 0, 0], "offsets": [0, 1, 2, 3]},
        # two leaves (:212-323)
        {"cite": "tstQueryTreeDegenerate.cpp:240-245", "leaves": [p0, p1], "kind": "box",
         "queries": [E], "indices": [], "offsets": [0, 0]},
        {"cite": "tstQueryTreeDegenerate.cpp:248-252", "leaves": [p0, p1], "kind": "box",
         "queries": [unit], "indices": [1, 0], "offsets": [0, 2]},
        {"cite": "tstQueryTreeDegenerate.cpp:255-259", "leaves": [p0, p1], "kind": "box",
         "queries": [[.5, .5, .5, 1.5, 1.5, 1.5]], "indices": [1], "offsets": [0, 1]},
        {"cite": "tstQueryTreeDegenerate.cpp:262-267", "leaves": [p0, p1], "kind": "box",
         "queries": [E, E], "indices": [], "offsets": [0, 0, 0]},
        {"cite": "tstQueryTreeDegenerate.cpp:270-275", "leaves": [p0, p1], "kind": "box",
         "queries": [E, p0], "indices": [0], "offsets": [0, 0, 1]},
        {"cite": "tstQueryTreeDegenerate.cpp:314-320", "leaves": [p0, p1], "kind": "nearest",
         "queries": [[0, 0, 0, 2], [1, 0, 0, 4]], "indices": [0, 1, 0, 1], "offsets": [0, 2, 4]},
        # duplicated leaves (:325-361)
        {"cite": "tstQueryTreeDegenerate.cpp:342-359", "leaves": [p0, p1, p1, p1], "kind": "sphere",
         "queries": [[0, 0, 0, 1], [1, 1, 1, 1], [.5, .5, .5, 1]],
         "indices": [0, 1, 2, 3, 0, 1, 2, 3], "offsets": [0, 1, 4, 8]},
        # buffer optimisation (tstQueryTreeTraversalPolicy.cpp:32-130)
        {"cite": "tstQueryTreeTraversalPolicy.cpp:43-60", "leaves": [p0, [1, 0, 0, 1, 0, 0], [2, 0, 0, 2, 0, 0], [3, 0, 0, 3, 0, 0]],
         "kind": "box", "queries": [E, [0, 0, 0, 3, 3, 3], E], "indices": [0, 1, 2, 3], "offsets": [0, 0, 4, 4],
         "buffer_sizes_ok": [0, -4, 5, -5, 1], "buffer_sizes_throw": [-1]},
        # unsorted predicates (:132-202)
        {"cite": "tstQueryTreeTraversalPolicy.cpp:152-174", "leaves": [p0, p1, [2, 2, 2, 2, 2, 2], [3, 3, 3, 3, 3, 3]],
         "kind": "box", "queries": [[2, 2, 2, 3, 3, 3], [0, 0, 0, 1, 1, 1]], "indices": [2, 3, 0, 1], "offsets": [0, 2, 4]},
        {"cite": "tstQueryTreeTraversalPolicy.cpp:177-199", "leaves": [p0, p1, [2, 2, 2, 2, 2, 2], [3, 3, 3, 3, 3, 3]],
         "kind": "nearest", "queries": [[2.5, 2.5, 2.5, 2], [.5, .5, .5, 2]], "indices": [2, 3, 0, 1], "offsets": [0, 2, 4]},
    ]
    return cases


def crs_query_impl():
    """test/tstDetailsCrsGraphWrapperImpl.cpp:49-101: predicate i reports
    values 0..i-1; two-pass CRS with hard preallocation 2(n+1)."""
    n = 10
    offsets, indices = [0], []
    for i in range(n):
        indices.extend(range(i))
        offsets.append(len(indices))
    return {"n": n, "buffer_size": 2 * (n + 1), "offsets": offsets, "indices": indices}


def neighbor_lists(root):
    """test/tstNeighborList.cpp:109-171: full neighbor lists (offsets,
    indices) of four points on the diagonal for several radii, and the
    degenerate empty / single-point clouds with an infinite radius.  The
    reference compares rows as multisets."""
    src = _read(root, "test/tstNeighborList.cpp")
    body = src[src.index("BOOST_AUTO_TEST_CASE_TEMPLATE(find_neighbor_list,"):]
    pts_txt = body[body.index("std::vector<Point>{") + len("std::vector<Point>{"):body.index('"Test::four_points"')]
    points = [[float(v.rstrip("f")) for v in t.split(",")]
              for t in re.findall(r"\{([-0-9.f, ]+)\}", pts_txt)]
    cases = []
    pat = re.compile(r"ARBORX_TEST_NEIGHBOR_LIST\(\s*exec_space,\s*points,\s*\(Coordinate\)([0-9.]+),\s*"
                     r"\(std::vector<int>\{([0-9, ]*)\}\),\s*\(std::vector<int>\{([0-9, ]*)\}\)\)", re.S)
    for r, off, idx in pat.findall(body):
        cases.append({"radius": float(r),
                      "offsets": [int(x) for x in off.replace(" ", "").split(",") if x],
                      "indices": [int(x) for x in idx.replace(" ", "").split(",") if x]})
    assert len(points) == 4 and len(cases) == 4, (points, cases)
    return {"cite": "test/tstNeighborList.cpp:109-171", "points": points, "cases": cases,
            "degenerate": [{"n": 0, "offsets": [0], "indices": []},
                           {"n": 1, "offsets": [0, 0], "indices": []}]}


def _f32_expr(txt):
    """Value of a test's float expression like -.5f*sqrtf_2 or 2*sqrtf_3,
    evaluated in float32 as the test does (sqrtf_k = std::sqrt(k.f))."""
    import numpy as np

    env = {"sqrtf_%d" % k: np.sqrt(np.float32(k)) for k in (2, 3, 5)}
    t = txt.strip().replace("f", "") if "sqrtf" not in txt else txt.strip()
    t = re.sub(r"(?<![a-z_])([0-9]*\.?[0-9]+)f", r"\1", t)
    v = eval(t, {"np": np}, {k: v for k, v in env.items()})
    return float(np.float32(v))


def rays(root):
    """test/tstRay.cpp:17-275 (intersects_box, ray_box_intersection with a
    1e-6 tolerance, ray_box_distance) against the unit box, and
    test/tstQueryTreeRay.cpp:62-265 (ten diagonal boxes; ordered results,
    empty and one-leaf trees).  Rays as written in the test (the library
    normalizes the direction)."""
    src = _read(root, "test/tstRay.cpp")
    num = r"[-0-9.]+"
    ray = r"Ray\{\{(%s), (%s), (%s)\}, \{(%s), (%s), (%s)\}\}" % ((num,) * 6)
    inter = [{"ray": [float(x) for x in m[1:]], "hit": m[0] == ""}
             for m in re.findall(r"BOOST_TEST\((!?)intersects\(" + ray + r", unit_box\)\);", src)]
    vals = []
    for m in re.finditer(r"ARBORX_TEST_RAY_BOX_INTERSECTION\(\(" + ray + r"\), unit_box, ?([^,]+), ([^)]+)\);", src):
        g = m.groups()
        vals.append({"ray": [float(x) for x in g[:6]], "t0": _f32_expr(g[6]), "t1": _f32_expr(g[7])})
    for m in re.finditer(r"ARBORX_TEST_RAY_BOX_NO_INTERSECTION\(\(" + ray + r"\), unit_box\);", src):
        vals.append({"ray": [float(x) for x in m.groups()], "hit": False})
    dist = []
    for m in re.finditer(r"BOOST_TEST\(distance\(" + ray + r", unit_box\) == ([^)]+)\);", src):
        g = m.groups()
        d = g[6].strip()
        dist.append({"ray": [float(x) for x in g[:6]], "distance": "inf" if d == "inf" else float(d.rstrip("f"))})
    assert len(inter) >= 40 and len(vals) >= 40 and len(dist) == 3, (len(inter), len(vals), len(dist))
    n = 10
    boxes = [[i, i, i, i + 1, i + 1, i + 1] for i in range(n)]
    return {"cite": "test/tstRay.cpp:17-275, test/tstQueryTreeRay.cpp:62-265",
            "unit_box": [0, 0, 0, 1, 1, 1], "intersects_box": inter, "intersection": vals,
            "distance": dist,
            "tree_boxes": boxes,
            "tree_intersects": {"ray": [0, 0, 0, .1, .1, .1], "indices": list(range(n))},
            "tree_ordered": [{"ray": [0, 0, 0, 1 / n, 1 / n, 1 / n], "indices": list(range(n))},
                             {"ray": [n, n, n, -1 / n, -1 / n, -1 / n], "indices": list(range(n - 1, -1, -1))}],
            "tree_nearest": {"ray": [0, 0, 0, .15, .1, 0], "k": 1, "indices": [0]},
            "single_leaf": {"box": [0, 0, 0, 1, 1, 1],
                            "rays": [[0, 0, 0, 1, 1, 1], [4, 5, 6, 7, 8, 9]], "offsets": [0, 1, 1],
                            "indices": [0]}}



def kdops(root):
    """test/tstGeometryIntersects.cpp:384-571 (KDOP<3, k> for k = 6, 14, 18,
    26: KDOP-KDOP and KDOP-box against the empty KDOP / box, and the two
    point-KDOP polytopes with their per-k expected answers) and
    test/tstQueryTreeIntersectsKDOP.cpp:26-91 (13 points, a KDOP<3, 18>
    predicate; empty predicate list).  Points in each polytope are the
    expand() calls in order."""
    src = _read(root, "test/tstGeometryIntersects.cpp")
    body = src[src.index("BOOST_AUTO_TEST_CASE_TEMPLATE(intersects_point_kdop, KDOP_t, KDOP_3D_types)"):]
    body = body[:body.index("\n}\n") + 3]
    flat = re.sub(r"\s+", " ", body)
    blocks = flat.split("KDOP_t x;")[1:]
    num = r"[-0-9.]+"
    pt = r"Point\{(%s), (%s), (%s)\}" % (num, num, num)
    polytopes = []
    for blk in blocks:
        expands = [[float(v) for v in m] for m in re.findall(r"expand\(x, " + pt + r"\);", blk)]
        checks = []
        for neg, x, y, z, cond in re.findall(
                r"BOOST_TEST\((!?)sym_intersects\(" + pt + r", x\)(?: == \(?([a-z_0-9| ]+)\)?)?\);", blk):
            expect = {}
            for k, flag in ((6, "is_kdop_3_6"), (14, "is_kdop_3_14"), (18, "is_kdop_3_18"), (26, None)):
                if cond:
                    val = any(c.strip() == flag for c in cond.split("||"))
                else:
                    val = neg == ""
                expect[str(k)] = val
            checks.append({"point": [float(x), float(y), float(z)], "expected": expect})
        polytopes.append({"expand": expands, "checks": checks})
    assert [blk.count("sym_intersects(") for blk in blocks] == [len(p["checks"]) for p in polytopes]
    assert [(len(p["expand"]), len(p["checks"])) for p in polytopes] == [(0, 1), (10, 9), (9, 9)]
    qsrc = _read(root, "test/tstQueryTreeIntersectsKDOP.cpp")
    prims = [[float(v) for v in m] for m in re.findall(r"\{\{(%s), (%s), (%s)\}\}, // \d+" % (num, num, num), qsrc)]
    qexp = [[float(v) for v in m] for m in re.findall(r"expand\(x, " + pt + r"\);", qsrc)]
    sol = re.findall(r"make_reference_solution<int>\(\{([0-9, ]*)\}, \{([0-9, ]*)\}\)", qsrc)
    ints = lambda t: [int(v) for v in t.replace(" ", "").split(",") if v]
    assert len(prims) == 13 and len(qexp) == 10 and len(sol) == 2, (len(prims), len(qexp), sol)
    unit = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    return {"cite": "test/tstGeometryIntersects.cpp:384-571, test/tstQueryTreeIntersectsKDOP.cpp:26-91",
            # intersects_kdop_kdop_3D / intersects_kdop_box_3D (:440-472): the
            # empty KDOP meets nothing; after expanding by the three unit
            # points it meets itself and the unit box, never an empty KDOP or
            # the empty Box{}
            "kdop_kdop": {"expand": unit, "self_before": False, "self_after": True,
                          "empty_after": False},
            "kdop_box": {"expand": unit, "unit_box": [0, 0, 0, 1, 1, 1],
                         "before": {"empty": False, "unit": False},
                         "after": {"empty": False, "unit": True}},
            "point_kdop": polytopes,
            "tree": {"points": prims, "kdop18_expand": qexp,
                     "empty": {"indices": ints(sol[0][0]), "offsets": ints(sol[0][1])},
                     "query": {"indices": ints(sol[1][0]), "offsets": ints(sol[1][1])}}}


def _geometry_literal(txt, env):
    """A geometry argument of a reference test: Box{}, Box{{{..}}, {{..}}},
    Point{..} / Point{{..}}, or a named constant of the test case."""
    import math

    t = txt.strip()
    if t in env:
        return env[t]
    nums = [float(x) for x in re.findall(r"-?[0-9]*\.?[0-9]+(?:e-?[0-9]+)?", t)]
    if t.startswith("Box{}"):
        return ("box", "empty")
    if t.startswith("Box"):
        assert len(nums) == 6, t
        return ("box", nums)
    if t.startswith("Point"):
        assert len(nums) == 3, t
        return ("point", nums)
    raise ValueError(t + " " + str(math.pi))


def _split_args(call):
    depth, cur, out = 0, "", []
    for ch in call:
        if ch in "({":
            depth += 1
        elif ch in ")}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return out


def geometry(root):
    """test/tstGeometryIntersects.cpp:44-126 (point-box, box-box, sphere-point,
    sphere-box; both argument orders must agree, as sym_intersects checks)
    and test/tstGeometryDistance.cpp:39-67 (point-point and point-box
    distances, compared exactly with float std::sqrt)."""
    src = _read(root, "test/tstGeometryIntersects.cpp")
    cases = []
    for name, env in (("intersects_point_box", {"point": ("point", [1.0, 1.0, 1.0])}),
                      ("intersects_box_box", {"box": ("box", [0, 0, 0, 1, 1, 1])}),
                      ("intersects_sphere_point", {"sphere": ("sphere", [0, 0, 0, 1.0])}),
                      ("intersects_sphere_box", {"sphere": ("sphere", [0, 0, 0, 1.0])})):
        body = src[src.index("BOOST_AUTO_TEST_CASE_TEMPLATE(" + name + ","):]
        body = body[:body.index("\n}\n")]
        flat = re.sub(r"\s+", " ", body)
        for m in re.finditer(r"(?:static_assert|BOOST_TEST)\( ?(!?)sym_intersects\(", flat):
            i = m.end()
            depth, j = 1, i
            while depth:
                depth += {"(": 1, ")": -1}.get(flat[j], 0)
                j += 1
            a, b = _split_args(flat[i:j - 1])
            cases.append({"a": _geometry_literal(a, env), "b": _geometry_literal(b, env),
                          "expected": m.group(1) == ""})
    assert len(cases) == 4 + 13 + 5 + 2, len(cases)
    dsrc = _read(root, "test/tstGeometryDistance.cpp")
    dist = []
    body = dsrc[dsrc.index("BOOST_AUTO_TEST_CASE_TEMPLATE(distance_point_point,"):
                dsrc.index("BOOST_AUTO_TEST_CASE_TEMPLATE(distance_point_sphere,")]
    flat = re.sub(r"\s+", " ", body)
    env = {"box": ("box", [0, 0, 0, 1, 1, 1])}
    for m in re.finditer(r"BOOST_TEST\(sym_distance\((.*?)\) == (std::sqrt\(\(Coordinate\)([0-9]+)\)|[0-9]+)\);", flat):
        a, b = _split_args(m.group(1))
        want = {"sqrt_of": int(m.group(3))} if m.group(3) else {"value": float(m.group(2))}
        dist.append({"a": _geometry_literal(a, env), "b": _geometry_literal(b, env), "expected": want})
    assert len(dist) == 6, len(dist)
    return {"cite": "test/tstGeometryIntersects.cpp:44-126, test/tstGeometryDistance.cpp:39-67",
            "intersects": cases, "distance": dist}


def expand_half_to_full(root):
    """test/tstDetailsExpandHalfToFull.cpp:48-80."""
    src = _read(root, "test/tstDetailsExpandHalfToFull.cpp")
    body = src[src.index("BOOST_AUTO_TEST_CASE_TEMPLATE(expand_half_to_full,"):]
    flat = re.sub(r"\s+", " ", body)
    vec = r"\(std::vector<int>\{([0-9, ]*)\}\)"
    ints = lambda t: [int(v) for v in t.replace(" ", "").split(",") if v]
    cases = [{"offsets_in": ints(a), "indices_in": ints(b), "offsets_out": ints(c), "indices_out": ints(d)}
             for a, b, c, d in re.findall(r"ARBORX_TEST_EXPAND_HALF_TO_FULL\( ?exec_space, " + vec + ", " + vec
                                          + ", " + vec + ", " + vec + r"\)", flat)]
    assert len(cases) == 5, len(cases)
    return {"cite": "test/tstDetailsExpandHalfToFull.cpp:48-80", "cases": cases}

def main(root):
    data = {
        "source": "ArborX 2.1.99 test sources (read as text)",
        "morton": morton_kats(root),
        "karras": karras_example(root),
        "assign_morton_codes": assign_morton_codes(root),
        "degenerate": degenerate_cases(),
        "crs_query_impl": crs_query_impl(),
        "neighbor_lists": neighbor_lists(root),
        "rays": rays(root),
        "kdops": kdops(root),
        "geometry": geometry(root),
        "expand_half_to_full": expand_half_to_full(root),
        "stack_capacity": {"cite": "tstQueryTreeDegenerate.cpp:367-446", "n": 4096},
        "manufactured_grid": {"cite": "tstQueryTreeManufacturedSolution.cpp:64-269", "nx": 11, "L": 100.0},
    }
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(out, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
