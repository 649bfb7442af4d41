"""Neighbor lists (src/spatial/detail/ArborX_NeighborList.hpp:47-188) and
expandHalfToFull (ArborX_ExpandHalfToFull.hpp:23-69): the reference's golden
cases (rows as multisets, as its tests compare them), then exact rows on
random clouds: the full row is the spatial query's row without the point
itself, the half row keeps the points whose leaf comes earlier in Morton
order, and half + expansion gives the full rows as multisets."""

import numpy as np
import pytest
import torch

from oracle import oracle as o
from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rows(off, ind):
    off = off.cpu().numpy() if hasattr(off, "cpu") else off
    ind = ind.cpu().numpy() if hasattr(ind, "cpu") else ind
    return [ind[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


def test_neighbor_list_golden(ax, golden):
    nl = golden["neighbor_lists"]
    pts = cuda(np.asarray(nl["points"], np.float32))
    for case in nl["cases"]:
        want = [sorted(r) for r in rows(np.asarray(case["offsets"]), np.asarray(case["indices"], np.int32))]
        full = [sorted(r) for r in rows(*ax.find_full_neighbor_list(pts, case["radius"]))]
        assert full == want
        ho, hi = ax.find_half_neighbor_list(pts, case["radius"])
        expanded = [sorted(r) for r in rows(*ax.expand_half_to_full(ho, hi))]
        assert expanded == want
    for d in nl["degenerate"]:
        p = cuda(np.zeros((d["n"], 3), np.float32))
        off, ind = ax.find_full_neighbor_list(p, float("inf"))
        assert off.cpu().numpy().tolist() == d["offsets"] and ind.numel() == 0
        ho, hi = ax.find_half_neighbor_list(p, float("inf"))
        off, ind = ax.expand_half_to_full(ho, hi)
        assert off.cpu().numpy().tolist() == d["offsets"] and ind.numel() == 0


@pytest.mark.parametrize("n,r", [(100, 0.3), (20000, 0.05), (200000, 0.02)])
def test_neighbor_lists_exact_rows(ax, n, r):
    p = uniform_points(n, 300 + n)
    p[5:9] = p[4]  # duplicates
    pts = cuda(p)
    ref = o.OracleTree(p)
    leaf_pos = np.empty(n, np.int64)
    leaf_pos[ref.leaves["value"]] = np.arange(n)
    sph = np.concatenate([p, np.full((n, 1), r, np.float32)], axis=1)
    so, si = ref.spatial(o.KIND_SPHERE, sph)
    spatial_rows = rows(so, si)
    full = rows(*ax.find_full_neighbor_list(pts, r))
    half = rows(*ax.find_half_neighbor_list(pts, r))
    for i in range(n):
        assert full[i] == [q for q in spatial_rows[i] if q != i]
        assert half[i] == [q for q in spatial_rows[i] if leaf_pos[q] < leaf_pos[i]]
    ho, hi = ax.find_half_neighbor_list(pts, r)
    exp = rows(*ax.expand_half_to_full(ho, hi))
    mirrored = [[] for _ in range(n)]
    for k in range(n):
        for q in half[k]:
            mirrored[q].append(k)
    for i in range(n):
        assert exp[i] == half[i] + sorted(mirrored[i])
        assert sorted(exp[i]) == sorted(full[i])
    assert ax.device_errors() == 0
