"""The reference's geometry and half-to-full known answers through the GPU
path: one-value trees and brute force (test/tstGeometryIntersects.cpp:44-126,
test/tstGeometryDistance.cpp:39-67) and abx_expand_half_to_full
(test/tstDetailsExpandHalfToFull.cpp:48-80)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FLT_MAX = np.float32(3.40282347e38)


def geometry(g):
    kind, v = g
    if kind == "box" and v == "empty":
        return "box", np.array([[FLT_MAX] * 3 + [-FLT_MAX] * 3], np.float32)
    return kind, np.asarray([v], np.float32)


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_geometry_golden_on_gpu(ax, golden):
    g = golden["geometry"]
    for c in g["intersects"]:
        for a, b in ((c["a"], c["b"]), (c["b"], c["a"])):
            vk, vals = geometry(a)
            pk, pred = geometry(b)
            if vk == "sphere":
                continue
            if pk == "point":
                pk, pred = "box", np.concatenate([pred, pred], axis=1)
            kind = ax.SPHERE if pk == "sphere" else ax.BOX
            vkind = ax.BOX if vk == "box" else ax.POINT
            for index in (ax.BVH(cuda(vals), kind=vkind), ax.BruteForce(cuda(vals), kind=vkind)):
                ind, off = ax.query(index, ax.intersects(cuda(pred), kind))
                assert bool(off[-1].item()) == c["expected"], (c, type(index).__name__)
    for c in g["distance"]:
        _, q = geometry(c["a"])
        bk, vals = geometry(c["b"])
        e = c["expected"]
        want = np.sqrt(np.float32(e["sqrt_of"])) if "sqrt_of" in e else np.float32(e["value"])
        vkind = ax.BOX if bk == "box" else ax.POINT
        for index in (ax.BVH(cuda(vals), kind=vkind), ax.BruteForce(cuda(vals), kind=vkind)):
            ind, off, dist = ax.query(index, ax.nearest(cuda(q), 1), with_distances=True)
            assert dist.cpu().numpy()[0] == want, c


def test_expand_half_to_full_golden_on_gpu(ax, golden):
    for c in golden["expand_half_to_full"]["cases"]:
        off, ind = ax.expand_half_to_full(torch.tensor(c["offsets_in"], dtype=torch.int32).cuda(),
                                          torch.tensor(c["indices_in"], dtype=torch.int32).cuda())
        off, ind = off.cpu().tolist(), ind.cpu().tolist()
        assert off == c["offsets_out"]
        rows = [sorted(ind[off[i]:off[i + 1]]) for i in range(len(off) - 1)]
        want = [sorted(c["indices_out"][off[i]:off[i + 1]]) for i in range(len(off) - 1)]
        assert rows == want
