"""Request loop (abx_server_*): every request's results equal the same query
run alone through query(), whether it ran alone or coalesced with others
(mixed trees, kinds, k and radii, submitted concurrently)."""

import threading

import numpy as np
import pytest
import torch

from tests.helpers import uniform_points

pytestmark = pytest.mark.gpu


def _direct(ax, bvh, kind, rows, k):
    q = torch.from_numpy(np.ascontiguousarray(rows)).cuda()
    if kind == "nearest":
        i, o, d = ax.query(bvh, ax.nearest(q, k), with_distances=True)
        return i.cpu().numpy(), o.cpu().numpy(), d.cpu().numpy()
    i, o = ax.query(bvh, ax.intersects(q))
    return i.cpu().numpy(), o.cpu().numpy()


def _same(a, b):
    return len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


def _requests(rng, ntrees, count):
    reqs = []
    for _ in range(count):
        t = int(rng.integers(0, ntrees))
        nq = int(np.floor(10 ** rng.uniform(0, 3.5)))
        if rng.random() < 0.5:
            reqs.append((t, "nearest", rng.random((nq, 3), dtype=np.float32), int(rng.choice([1, 8, 32]))))
        else:
            c = rng.random((nq, 3), dtype=np.float32)
            r = rng.uniform(0.01, 0.05, (nq, 1)).astype(np.float32)
            reqs.append((t, "intersects", np.concatenate([c, r], axis=1), 0))
    return reqs


def _submit(srv, tids, req):
    t, kind, rows, k = req
    if kind == "nearest":
        return srv.submit_nearest(tids[t], rows, k)
    return srv.submit_intersects(tids[t], rows)


def test_results_alone_and_in_a_mix_are_identical(ax):
    trees = [ax.BoundingVolumeHierarchy(torch.from_numpy(uniform_points(n, 40 + n)).cuda())
             for n in (1000, 50000, 300000)]
    srv = ax.Server(workers=4, max_batch_queries=20000)
    tids = [srv.add_tree(b) for b in trees]
    reqs = _requests(np.random.default_rng(4), len(trees), 60)
    # alone: one request in flight at a time
    alone = []
    for req in reqs:
        alone.append(srv.result(_submit(srv, tids, req)))
    # in a mix: all submitted at once from 4 threads, then collected
    tickets = [None] * len(reqs)

    def submitter(j0):
        for j in range(j0, len(reqs), 4):
            tickets[j] = _submit(srv, tids, reqs[j])

    th = [threading.Thread(target=submitter, args=(j,)) for j in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    mixed = [srv.result(t) for t in tickets]
    st = srv.stats()
    assert st["batches"] < 2 * len(reqs)  # some coalescing happened
    for req, a, m in zip(reqs, alone, mixed):
        assert _same(a, m)
        t, kind, rows, k = req
        assert _same(a, _direct(ax, trees[t], kind, rows, k))
    assert st["completed_requests"] == 2 * len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()
    assert ax.device_errors() == 0


def test_server_rejects_bad_requests(ax):
    srv = ax.Server(workers=1)
    with pytest.raises(ax.SearchException):
        srv.submit_nearest(0, np.zeros((1, 3), np.float32), 1)  # no tree yet
    b = ax.BoundingVolumeHierarchy(torch.from_numpy(uniform_points(100, 1)).cuda())
    t = srv.add_tree(b)
    i, o, d = srv.result(srv.submit_nearest(t, np.zeros((0, 3), np.float32), 4))
    assert o.tolist() == [0] and i.size == 0
    srv.close()
