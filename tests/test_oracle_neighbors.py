"""findHalfNeighborList by the reference's HalfTraversal restated step for
step in the oracle (ArborX_HalfTraversal.hpp:23-75, ArborX_NeighborList.hpp:
47-111), against the reference's neighbor-list test and against the rows
this library computes: the sphere walk of each point keeping the leaves
before its own (the rows the GPU tests compare with)."""

import numpy as np
import pytest

from oracle import oracle as o
from tests.helpers import uniform_points


def _rows(off, ind):
    return [ind[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


def test_restated_half_traversal_golden(golden):
    """test/tstNeighborList.cpp:109-171: a half list and its mirror give the
    full lists of four points on the diagonal (multisets, as the test)."""
    nl = golden["neighbor_lists"]
    pts = np.asarray(nl["points"], np.float32)
    tree = o.OracleTree(pts)
    for case in nl["cases"]:
        half = _rows(*tree.half_neighbors(case["radius"]))
        full = [list(r) for r in half]
        for p, row in enumerate(half):
            for q in row:
                full[q].append(p)
        want = [sorted(case["indices"][case["offsets"][i]:case["offsets"][i + 1]]) for i in range(4)]
        assert [sorted(r) for r in full] == want
    for d in nl["degenerate"]:
        t = o.OracleTree(np.zeros((d["n"], 3), np.float32))
        off, ind = t.half_neighbors(1.0)
        assert off.tolist() == d["offsets"] and ind.size == 0


@pytest.mark.parametrize("n,r", [(2, 10.0), (300, 0.2), (20000, 0.04)])
def test_restated_half_traversal_equals_filtered_sphere_walk(n, r):
    """Run by increasing leaf position, the reference's half traversal lists
    each row's earlier leaves in Morton order: the same rows, order included,
    as the sphere walk that keeps the leaves before the point's own."""
    p = uniform_points(n, 700 + n)
    p[n // 3: n // 3 + min(5, n // 3)] = p[0]  # duplicates
    tree = o.OracleTree(p)
    leaf_pos = np.empty(n, np.int64)
    leaf_pos[tree.leaves["value"]] = np.arange(n)
    so, si = tree.spatial(o.KIND_SPHERE, np.concatenate([p, np.full((n, 1), r, np.float32)], 1))
    want = [[q for q in row if leaf_pos[q] < leaf_pos[i]] for i, row in enumerate(_rows(so, si))]
    assert _rows(*tree.half_neighbors(r)) == want
