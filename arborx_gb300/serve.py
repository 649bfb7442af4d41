"""Python face of the request loop (abx_server_* in include/arborx_gb300.h).

    srv = Server(workers=4)
    t = srv.add_tree(bvh)
    ticket = srv.submit_nearest(t, points_np, k=8)
    indices, offsets, distances = srv.result(ticket)

Queries are host numpy arrays (the server copies them); results come back as
host numpy arrays.  Requests submitted while others run are coalesced per
tree and kind and overlap on the device (continuous batching)."""

import ctypes

import numpy as np

from . import _lib
from ._lib import REQ_INTERSECTS, REQ_NEAREST, RequestC, ServerConfigC, ServerStatisticsC, check


class Server:
    def __init__(self, workers=4, max_inflight_bytes=8 << 30, max_batch_queries=1 << 20,
                 l2_persist=False):
        L = _lib.load()
        self._h = ctypes.c_void_p()
        cfg = ServerConfigC(workers, 1 if l2_persist else 0, max_inflight_bytes, max_batch_queries)
        check(L.abx_server_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._trees = []
        self._meta = {}

    def close(self):
        if self._h:
            _lib.load().abx_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_tree(self, bvh):
        tid = ctypes.c_int32()
        check(_lib.load().abx_server_add_tree(self._h, bvh._h, ctypes.byref(tid)))
        self._trees.append(bvh)  # the tree outlives the server's use of it
        return tid.value

    def _submit(self, tree, kind, rows, k):
        q = np.ascontiguousarray(rows, dtype=np.float32)
        req = RequestC(tree, kind, q.ctypes.data, q.shape[0], int(k), 0)
        ticket = ctypes.c_int64()
        check(_lib.load().abx_server_submit(self._h, ctypes.byref(req), ctypes.byref(ticket)))
        self._meta[ticket.value] = (kind, q.shape[0])
        return ticket.value

    def submit_nearest(self, tree, points, k):
        """nearest(point, k) for every row of points [nq, 3]."""
        return self._submit(tree, REQ_NEAREST, np.asarray(points).reshape(-1, 3), k)

    def submit_intersects(self, tree, spheres):
        """intersects(sphere) for every row of spheres [nq, 4] (x, y, z, r)."""
        return self._submit(tree, REQ_INTERSECTS, np.asarray(spheres).reshape(-1, 4), 0)

    def wait(self, ticket):
        """(number of results, latency in ms) once the request completed."""
        nres = ctypes.c_int64()
        lat = ctypes.c_double()
        check(_lib.load().abx_server_wait(self._h, ticket, ctypes.byref(nres), ctypes.byref(lat)))
        return nres.value, lat.value

    def result(self, ticket):
        """(indices, offsets[, distances]) of a completed request (nearest
        requests include distances); releases the request."""
        kind, nq = self._meta.pop(ticket)
        nres, _ = self.wait(ticket)
        off = np.empty(nq + 1, np.int32)
        idx = np.empty(max(nres, 1), np.int32)
        dist = np.empty(max(nres, 1), np.float32) if kind == REQ_NEAREST else None
        check(_lib.load().abx_server_result(self._h, ticket, off.ctypes.data, idx.ctypes.data,
                                            dist.ctypes.data if dist is not None else None))
        if dist is not None:
            return idx[:nres], off, dist[:nres]
        return idx[:nres], off

    def stats(self):
        st = ServerStatisticsC()
        check(_lib.load().abx_server_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStatisticsC._fields_}

    def reset_stats(self):
        check(_lib.load().abx_server_reset_stats(self._h))
