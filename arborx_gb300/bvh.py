"""Python mirror of the ArborX BVH interface over the C ABI.

Mirrors (reference paths relative to the ArborX source tree):
  BoundingVolumeHierarchy   src/spatial/ArborX_LinearBVH.hpp:57-142
  query(tree, preds, ...)   src/spatial/ArborX_CrsGraphWrapper.hpp:22-34
  intersects / nearest      src/spatial/detail/ArborX_Predicates.hpp:57-142
  make_intersects/_nearest  src/spatial/detail/ArborX_PredicateHelpers.hpp:92-206
  TraversalPolicy           src/spatial/detail/ArborX_TraversalPolicy.hpp:19-47
Tensors are torch CUDA tensors (PyTorch is only the device-memory and stream
plumbing); every computation is a kernel of libarborx_gb300.so.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import BOX, KDOP6, KDOP14, KDOP18, KDOP26, KDOP_NDIR, POINT, RAY, SPHERE, TraversalPolicyC, check


def version():
    return _lib.load().abx_version().decode()


def _stream(space):
    if space is None:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(space, torch.cuda.Stream):
        return ctypes.c_void_p(space.cuda_stream)
    return ctypes.c_void_p(int(space))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else ctypes.c_void_p(0)


def _as_rows(t, cols, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != torch.float32:
        t = t.to(torch.float32)
    t = t.contiguous()
    if t.numel() % cols != 0:
        raise ValueError("%s: expected rows of %d floats, got shape %s" % (name, cols, tuple(t.shape)))
    return t.view(-1, cols)


class _CrsOwner:
    """Owns an abx_crs; freed when the last view of its arrays goes away."""

    def __init__(self, handle):
        self.handle = handle

    def __del__(self):
        if self.handle:
            try:
                _lib.load().abx_crs_destroy(self.handle)
            except Exception:  # interpreter shutdown
                pass
            self.handle = None


class _DeviceArray:
    def __init__(self, owner, ptr, n, typestr):
        self._owner = owner
        self.__cuda_array_interface__ = {
            "shape": (int(n),),
            "typestr": typestr,
            "data": (int(ptr), False),
            "version": 2,
        }


def _view(owner, ptr, n, dtype):
    if n == 0 or not ptr:
        return torch.empty(0, dtype=dtype, device="cuda")
    typestr = {torch.int32: "<i4", torch.float32: "<f4"}[dtype]
    return torch.as_tensor(_DeviceArray(owner, ptr, n, typestr), device="cuda")


class TraversalPolicy:
    """ArborX::Experimental::TraversalPolicy: buffer size 0 (two-pass), > 0
    (single pass, second pass on overflow), < 0 (single pass, overflow raises
    SearchException); predicate sorting on by default."""

    def __init__(self, buffer_size=0, sort_predicates=True):
        self._buffer_size = int(buffer_size)
        self._sort_predicates = bool(sort_predicates)

    def setBufferSize(self, buffer_size):  # noqa: N802 (ArborX spelling)
        self._buffer_size = int(buffer_size)
        return self

    def setPredicateSorting(self, sort_predicates):  # noqa: N802
        self._sort_predicates = bool(sort_predicates)
        return self

    def _c(self):
        return TraversalPolicyC(self._buffer_size, 1 if self._sort_predicates else 0)


def _columns(kind):
    """Floats per value of a geometry kind."""
    if kind in KDOP_NDIR:
        return 2 * KDOP_NDIR[kind]
    return {POINT: 3, BOX: 6, SPHERE: 4, RAY: 6}[kind]


def _kind_of(cols, what):
    """Geometry kind of a value width (6 columns: a box; KDOP<3, 6> needs an
    explicit kind)."""
    kind = {3: POINT, 4: SPHERE, 6: BOX, 14: KDOP14, 18: KDOP18, 26: KDOP26}.get(cols)
    if kind is None:
        raise ValueError("%s: no geometry has %d columns" % (what, cols))
    return kind


class Intersects:
    """Batch of intersects(geometry) predicates: spheres [nq,4] (cx cy cz r),
    boxes [nq,6] (min xyz, max xyz), rays [nq,6] or KDOP<3, k> [nq, k]
    (min of the k/2 directions, then max)."""

    def __init__(self, geometry, kind):
        self.kind = kind
        self.data = _as_rows(geometry, _columns(kind), "intersects geometry")

    def __len__(self):
        return self.data.shape[0]


class OrderedIntersects:
    """Batch of Experimental::ordered_intersects(Ray) predicates
    (ArborX_Predicates.hpp:103-125): rays [nq, 6] (origin xyz, direction
    xyz; the library normalizes the direction as the Ray constructor does).
    k > 0 keeps the first k hits per ray (nearest(Ray, k))."""

    def __init__(self, rays, k=0):
        self.data = _as_rows(rays, 6, "rays")
        self.k = int(k)

    def __len__(self):
        return self.data.shape[0]


def ordered_intersects(rays, k=0):
    return OrderedIntersects(rays, k)


def ray_intersects(rays):
    """intersects(Ray) for every row of rays [nq, 6]."""
    return Intersects(rays, RAY)


class Nearest:
    """Batch of nearest(point, k) predicates: points [nq,3] and k (int or an
    int32 CUDA tensor with one k per query)."""

    def __init__(self, points, k=1):
        self.data = _as_rows(points, 3, "nearest points")
        if isinstance(k, torch.Tensor):
            self.k = k.to(device=self.data.device, dtype=torch.int32).contiguous()
        else:
            self.k = int(k)

    def __len__(self):
        return self.data.shape[0]


def intersects(geometry, kind=None):
    """intersects(Sphere | Box | KDOP) predicates; the kind follows the number
    of columns (4 sphere, 6 box, 14 / 18 / 26 KDOP) unless given."""
    g = geometry
    if kind is None:
        kind = _kind_of(g.shape[-1], "intersects")
        if kind == POINT:
            raise ValueError("intersects: points are predicates as degenerate boxes [p, p]")
    return Intersects(g, kind)


def kdop_from(geometry, k, kind=None, space=None):
    """KDOP<3, k> (k = 6, 14, 18, 26) of every point [n, 3] or box [n, 6]:
    KDOP{} expanded by the geometry (abx_kdop_from_geometry).  Returns a
    float32 CUDA tensor [n, k]."""
    kk = {6: KDOP6, 14: KDOP14, 18: KDOP18, 26: KDOP26}[int(k)]
    if kind is None:
        kind = {3: POINT, 6: BOX}.get(geometry.shape[-1])
        if kind is None:
            raise ValueError("kdop_from: points [n, 3] or boxes [n, 6]")
    g = _as_rows(geometry, _columns(kind), "geometry")
    out = torch.empty((g.shape[0], int(k)), dtype=torch.float32, device=g.device)
    check(_lib.load().abx_kdop_from_geometry(_stream(space), kind, _ptr(g), g.shape[0], kk, _ptr(out)))
    return out


def nearest(points, k=1):
    return Nearest(points, k)


def make_intersects(points, r):
    """intersects(Sphere{p, r}) for every point (ArborX_PredicateHelpers.hpp:99-105)."""
    p = _as_rows(points, 3, "points")
    rr = torch.full((p.shape[0], 1), float(r), dtype=torch.float32, device=p.device)
    return Intersects(torch.cat([p, rr], dim=1), SPHERE)


def make_nearest(points, k):
    """nearest(p, k) for every point (ArborX_PredicateHelpers.hpp:114-119)."""
    return Nearest(points, k)


class BoundingVolumeHierarchy:
    """Tree over points [n,3], boxes [n,6] or KDOP<3, k> [n, k] (nodes then
    bounded by KDOPs too: BVH<MemorySpace, Value, IndexableGetter, KDOP>); the
    value of each leaf is its row index (ArborX's benchmark form
    BVH<MemorySpace, int, ...>)."""

    def __init__(self, values=None, space=None, kind=None):
        L = _lib.load()
        self._h = ctypes.c_void_p()
        if values is None:
            values = torch.empty((0, 3), dtype=torch.float32, device="cuda")
            kind = POINT
        if kind is None:
            kind = _kind_of(values.shape[-1], "values")
            if kind not in (POINT, BOX) and kind not in KDOP_NDIR:
                raise ValueError("values must be points, boxes or KDOPs")
        self.kind = kind
        self._stream = _stream(space)
        cols = _columns(kind)
        if (isinstance(values, torch.Tensor) and values.is_cuda and values.dtype == torch.float32
                and values.dim() == 2 and values.shape[1] == cols and not values.is_contiguous()):
            # any layout (access traits): read through the tensor's strides
            v = values
            vals = _lib.ValuesC(v.data_ptr(), v.stride(0), v.stride(1))
            check(L.abx_bvh_create_strided(self._stream, kind, vals, v.shape[0],
                                           ctypes.byref(self._h)))
        else:
            v = _as_rows(values, cols, "values")
            check(L.abx_bvh_create(self._stream, kind, _ptr(v), v.shape[0], ctypes.byref(self._h)))
        self._values = v  # kept until the build has consumed it

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().abx_bvh_destroy(h)
            except Exception:
                pass
            self._h = None

    def size(self):
        return int(_lib.load().abx_bvh_size(self._h))

    def empty(self):
        return self.size() == 0

    def bounds(self):
        """The root box as (min xyz, max xyz); waits for the build."""
        out = (ctypes.c_float * 6)()
        check(_lib.load().abx_bvh_bounds(self._h, out))
        return tuple(out)

    def export_nodes(self, space=None):
        """Node arrays in the reference layout: leaves int32 [n,2] (rope,
        value) and internal nodes int32 [n-1,8] (left_child, rope, then the
        box's 6 floats stored bit-for-bit)."""
        n = self.size()
        leaves = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        internal = torch.empty((max(n - 1, 0), 8), dtype=torch.int32, device="cuda")
        check(_lib.load().abx_bvh_export_nodes(self._h, _stream(space), _ptr(leaves), _ptr(internal)))
        return leaves, internal

    def query(self, predicates, policy=None, space=None, with_distances=False):
        return query(self, predicates, policy, space=space, with_distances=with_distances)

    def kdop_bounds(self):
        """The KDOP of the whole tree (KDOP trees); waits for the build."""
        out = (ctypes.c_float * (2 * KDOP_NDIR[self.kind]))()
        check(_lib.load().abx_bvh_kdop_bounds(self._h, out))
        return tuple(out)

    def save(self, path):
        """Write the tree to a file (abx_bvh_save)."""
        check(_lib.load().abx_bvh_save(self._h, str(path).encode()))

    @classmethod
    def load(cls, path, space=None):
        """A tree read back from a file written by save() (abx_bvh_load)."""
        t = cls.__new__(cls)
        t._h = ctypes.c_void_p()
        t._stream = _stream(space)
        check(_lib.load().abx_bvh_load(t._stream, str(path).encode(), ctypes.byref(t._h)))
        t.kind = int(_lib.load().abx_bvh_geometry(t._h))
        t._values = None
        return t


BVH = BoundingVolumeHierarchy


class BruteForce:
    """ArborX::BruteForce (src/spatial/ArborX_BruteForce.hpp:40-176): every
    predicate against every value.  Same query API as the tree; nearest results
    equal the tree's, intersects results come in ascending value order."""

    _prefix = "abx_brute"

    def __init__(self, values, space=None, kind=None):
        L = _lib.load()
        self._h = ctypes.c_void_p()
        if kind is None:
            kind = {3: POINT, 6: BOX}.get(values.shape[-1])
            if kind is None:
                raise ValueError("values must have 3 (point) or 6 (box) columns")
        self.kind = kind
        v = _as_rows(values, 3 if kind == POINT else 6, "values")
        check(L.abx_brute_create(_stream(space), kind, _ptr(v), v.shape[0], ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().abx_brute_destroy(h)
            except Exception:
                pass
            self._h = None

    def size(self):
        return int(_lib.load().abx_brute_size(self._h))

    def empty(self):
        return self.size() == 0

    def bounds(self):
        out = (ctypes.c_float * 6)()
        check(_lib.load().abx_brute_bounds(self._h, out))
        return tuple(out)

    def query(self, predicates, policy=None, space=None, with_distances=False):
        return query(self, predicates, policy, space=space, with_distances=with_distances)


def query(tree, predicates, policy=None, space=None, with_distances=False):
    """ArborX::query(tree, space, predicates, indices, offsets[, policy]).

    Returns (indices, offsets) as int32 CUDA tensors; nearest predicates with
    with_distances=True also return the float32 distances."""
    L = _lib.load()
    policy = policy or TraversalPolicy()
    s = _stream(space)
    h = ctypes.c_void_p()
    prefix = getattr(tree, "_prefix", "abx_bvh")
    if isinstance(predicates, Intersects):
        check(
            getattr(L, prefix + "_query_intersects")(
                tree._h, s, predicates.kind, _ptr(predicates.data), len(predicates), policy._c(),
                ctypes.byref(h),
            )
        )
    elif isinstance(predicates, Nearest):
        kt = predicates.k if isinstance(predicates.k, torch.Tensor) else None
        kv = 0 if kt is not None else predicates.k
        check(
            getattr(L, prefix + "_query_nearest")(
                tree._h, s, _ptr(predicates.data), len(predicates), _ptr(kt) if kt is not None else None,
                kv, policy._c(), 1 if with_distances else 0, ctypes.byref(h),
            )
        )
    elif isinstance(predicates, OrderedIntersects):
        if prefix != "abx_bvh":
            raise TypeError("ordered_intersects: tree queries only")
        check(L.abx_bvh_query_ordered_intersects(
            tree._h, s, _ptr(predicates.data), len(predicates), predicates.k, policy._c(),
            1 if with_distances else 0, ctypes.byref(h)))
        return _crs_result(h, with_distances)
    else:
        raise TypeError("predicates must be Intersects, Nearest or OrderedIntersects")
    return _crs_result(h, isinstance(predicates, Nearest) and with_distances)


def query_nearest_into(tree, queries, k, offsets, indices, distances=None, policy=None,
                       space=None):
    """nearest(point, k) into preallocated int32 offsets [nq + 1] and indices
    [nq * min(k, size)] (and float32 distances) with no host synchronisation:
    the call can be captured in a CUDA graph (torch.cuda.graph) and replayed."""
    policy = policy or TraversalPolicy()
    q = _as_rows(queries, 3, "queries")
    for t, name in ((offsets, "offsets"), (indices, "indices")):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.int32 and t.is_contiguous()):
            raise TypeError("%s must be a contiguous int32 CUDA tensor" % name)
    check(_lib.load().abx_bvh_query_nearest_into(
        tree._h, _stream(space), _ptr(q), q.shape[0], int(k), policy._c(), _ptr(offsets),
        _ptr(indices), _ptr(distances) if distances is not None else None))


def query_nearest_host(tree, queries, k, offsets, indices, distances=None, chunk=0, policy=None,
                       space=None):
    """nearest(point, k) with the queries [nq, 3] and the results in host
    memory (float32 / int32 CPU tensors; pinned for the copies to overlap):
    offsets [nq + 1], indices [nq * min(k, size)], distances optional.  The
    queries move to the device in chunks pipelined with the traversal and the
    copies back (abx_bvh_query_nearest_host)."""
    policy = policy or TraversalPolicy()
    for t, name, dt in ((queries, "queries", torch.float32), (offsets, "offsets", torch.int32),
                        (indices, "indices", torch.int32)):
        if not (isinstance(t, torch.Tensor) and not t.is_cuda and t.dtype == dt and t.is_contiguous()):
            raise TypeError("%s must be a contiguous %s CPU tensor" % (name, dt))
    if distances is not None and not (isinstance(distances, torch.Tensor) and not distances.is_cuda
                                      and distances.dtype == torch.float32 and distances.is_contiguous()):
        raise TypeError("distances must be a contiguous float32 CPU tensor")
    nq = queries.shape[0] if queries.dim() == 2 else queries.numel() // 3
    kk = min(max(int(k), 0), tree.size())
    if offsets.numel() < nq + 1 or indices.numel() < nq * kk or (
            distances is not None and distances.numel() < nq * kk):
        raise ValueError("query_nearest_host: output tensors too small")
    check(_lib.load().abx_bvh_query_nearest_host(
        tree._h, _stream(space), queries.data_ptr(), nq, int(k), policy._c(), int(chunk),
        offsets.data_ptr(), indices.data_ptr(), distances.data_ptr() if distances is not None else None))


def _neighbor_list(points, radius, half, space):
    p = _as_rows(points, 3, "points")
    h = ctypes.c_void_p()
    check(_lib.load().abx_find_neighbor_list(_stream(space), _ptr(p), p.shape[0], float(radius),
                                             1 if half else 0, ctypes.byref(h)))
    indices, offsets = _crs_result(h, False)
    return offsets, indices


def find_full_neighbor_list(points, radius, space=None):
    """ArborX::Experimental::findFullNeighborList (ArborX_NeighborList.hpp:
    113-186): (offsets, indices), row p = every other point within radius,
    in the tree's depth-first order."""
    return _neighbor_list(points, radius, False, space)


def find_half_neighbor_list(points, radius, space=None):
    """ArborX::Experimental::findHalfNeighborList (ArborX_NeighborList.hpp:
    47-111): (offsets, indices), row p = the points within radius whose leaf
    precedes p's in the tree's Morton order (each pair once)."""
    return _neighbor_list(points, radius, True, space)


def expand_half_to_full(offsets, indices, space=None):
    """ArborX::Details::expandHalfToFull (ArborX_ExpandHalfToFull.hpp:23-69):
    (offsets, indices) of the full list; row i = its half row, then the rows
    listing i in ascending order."""
    h = ctypes.c_void_p()
    o = offsets.to(torch.int32).contiguous()
    i = indices.to(torch.int32).contiguous()
    check(_lib.load().abx_expand_half_to_full(_stream(space), o.numel() - 1, _ptr(o), _ptr(i),
                                              ctypes.byref(h)))
    ind, off = _crs_result(h, False)
    return off, ind


def _crs_result(h, with_distances):
    L = _lib.load()
    owner = _CrsOwner(h)
    nq = L.abx_crs_num_queries(h)
    nres = L.abx_crs_num_results(h)
    offsets = _view(owner, L.abx_crs_offsets(h), nq + 1, torch.int32)
    indices = _view(owner, L.abx_crs_indices(h), nres, torch.int32)
    if with_distances:
        dist = _view(owner, L.abx_crs_distances(h), nres, torch.float32)
        return indices, offsets, dist
    return indices, offsets


def _offsets_array(offsets, name):
    o = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
    if o.ndim != 1 or o.size < 2:
        raise ValueError("%s must hold at least two entries" % name)
    return o


class Forest:
    """A batch of independent trees built together: tree t holds the rows
    values[offsets[t]:offsets[t + 1]] and is exactly the tree that
    BoundingVolumeHierarchy(values[offsets[t]:offsets[t + 1]]) builds (same
    node arrays, tree-local values).  Replaces the reference's loop of one
    BVH per subview (benchmarks/execution_space_instances/
    execution_space_instances_driver.cpp:187-233)."""

    def __init__(self, values, offsets, space=None, kind=None):
        L = _lib.load()
        self._h = ctypes.c_void_p()
        if kind is None:
            kind = {3: POINT, 6: BOX}.get(values.shape[-1])
            if kind is None:
                raise ValueError("values must have 3 (point) or 6 (box) columns")
        self.kind = kind
        v = _as_rows(values, 3 if kind == POINT else 6, "values")
        o = _offsets_array(offsets, "offsets")
        if o[-1] != v.shape[0]:
            raise ValueError("offsets[-1] must equal the number of values")
        self._offsets = o
        self._stream = _stream(space)
        check(L.abx_forest_create(self._stream, kind, _ptr(v), o.ctypes.data, o.size - 1,
                                  ctypes.byref(self._h)))
        self._values = v

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().abx_forest_destroy(h)
            except Exception:
                pass
            self._h = None

    def num_trees(self):
        return int(_lib.load().abx_forest_num_trees(self._h))

    def size(self, tree):
        return int(_lib.load().abx_forest_size(self._h, tree))

    def bounds(self, tree):
        out = (ctypes.c_float * 6)()
        check(_lib.load().abx_forest_bounds(self._h, tree, out))
        return tuple(out)

    def export_nodes(self, tree, space=None):
        """Node arrays of one tree, laid out like
        BoundingVolumeHierarchy.export_nodes."""
        n = self.size(tree)
        leaves = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        internal = torch.empty((max(n - 1, 0), 8), dtype=torch.int32, device="cuda")
        check(_lib.load().abx_forest_export_nodes(self._h, tree, _stream(space), _ptr(leaves),
                                                  _ptr(internal)))
        return leaves, internal

    def query(self, predicates, query_offsets, policy=None, space=None, with_distances=False):
        """Predicates predicates[query_offsets[t]:query_offsets[t + 1]] run on
        tree t.  Returns one CRS result over all queries with tree-local
        indices: (indices, offsets[, distances])."""
        L = _lib.load()
        policy = policy or TraversalPolicy()
        qo = _offsets_array(query_offsets, "query_offsets")
        if qo.size != self._offsets.size:
            raise ValueError("query_offsets needs one entry per tree plus one")
        if qo[-1] != len(predicates):
            raise ValueError("query_offsets[-1] must equal the number of predicates")
        s = _stream(space)
        h = ctypes.c_void_p()
        if isinstance(predicates, Intersects):
            check(L.abx_forest_query_intersects(self._h, s, predicates.kind, _ptr(predicates.data),
                                                qo.ctypes.data, policy._c(), ctypes.byref(h)))
            return _crs_result(h, False)
        if isinstance(predicates, Nearest):
            kt = predicates.k if isinstance(predicates.k, torch.Tensor) else None
            kv = 0 if kt is not None else predicates.k
            check(L.abx_forest_query_nearest(
                self._h, s, _ptr(predicates.data), qo.ctypes.data,
                _ptr(kt) if kt is not None else None, kv, policy._c(),
                1 if with_distances else 0, ctypes.byref(h)))
            return _crs_result(h, with_distances)
        raise TypeError("predicates must be Intersects or Nearest")


# ---------------------------------------------------------------------------
# Building blocks (the reference's Details functions)
# ---------------------------------------------------------------------------


def device_errors(space=None):
    bits = ctypes.c_uint32(0)
    check(_lib.load().abx_device_errors(_stream(space), ctypes.byref(bits)))
    return bits.value


def scene_bounds(values, kind=POINT, space=None):
    v = _as_rows(values, 3 if kind == POINT else 6, "values")
    out = torch.empty(6, dtype=torch.float32, device="cuda")
    check(_lib.load().abx_scene_bounds(_stream(space), kind, _ptr(v), v.shape[0], _ptr(out)))
    return out


def morton64(values, scene, kind=POINT, space=None):
    """Morton64 codes (uint64 bit patterns in an int64 tensor)."""
    v = _as_rows(values, {POINT: 3, BOX: 6, SPHERE: 4}[kind], "values")
    sc = scene.to(device="cuda", dtype=torch.float32).contiguous()
    out = torch.empty(v.shape[0], dtype=torch.int64, device="cuda")
    check(_lib.load().abx_morton64(_stream(space), kind, _ptr(v), v.shape[0], _ptr(sc), _ptr(out)))
    return out


def morton32(values, scene, kind=POINT, space=None):
    """Morton32 codes (uint32 bit patterns in an int32 tensor)."""
    v = _as_rows(values, {POINT: 3, BOX: 6, SPHERE: 4}[kind], "values")
    sc = scene.to(device="cuda", dtype=torch.float32).contiguous()
    out = torch.empty(v.shape[0], dtype=torch.int32, device="cuda")
    check(_lib.load().abx_morton32(_stream(space), kind, _ptr(v), v.shape[0], _ptr(sc), _ptr(out)))
    return out


def sort_u64(keys, space=None):
    """Stable sort of uint64 keys (int64 tensor, sorted in place); returns the
    permutation (int32 tensor)."""
    assert keys.dtype == torch.int64 and keys.is_cuda and keys.is_contiguous()
    perm = torch.empty(keys.numel(), dtype=torch.int32, device="cuda")
    check(_lib.load().abx_sort_u64(_stream(space), _ptr(keys), keys.numel(), _ptr(perm)))
    return perm


def sort_u32(keys, space=None):
    assert keys.dtype == torch.int32 and keys.is_cuda and keys.is_contiguous()
    perm = torch.empty(keys.numel(), dtype=torch.int32, device="cuda")
    check(_lib.load().abx_sort_u32(_stream(space), _ptr(keys), keys.numel(), _ptr(perm)))
    return perm


def generate_hierarchy(values, permutation, sorted_codes, kind=POINT, space=None):
    v = _as_rows(values, 3 if kind == POINT else 6, "values")
    n = v.shape[0]
    leaves = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    internal = torch.empty((max(n - 1, 0), 8), dtype=torch.int32, device="cuda")
    check(
        _lib.load().abx_generate_hierarchy(
            _stream(space), kind, _ptr(v), n, _ptr(permutation.contiguous()),
            _ptr(sorted_codes.contiguous()), _ptr(leaves), _ptr(internal),
        )
    )
    return leaves, internal


def exclusive_scan(values, space=None):
    v = values.to(torch.int32).contiguous()
    out = torch.empty(v.numel() + 1, dtype=torch.int32, device="cuda")
    check(_lib.load().abx_exclusive_scan_i32(_stream(space), _ptr(v), v.numel(), _ptr(out)))
    return out
