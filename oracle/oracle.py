"""Python front end of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the ArborX BoundingVolumeHierarchy hot
path (``oracle/abx_oracle.c``; each C function cites the reference file:line it
follows).  It is the CHECKER for the CUDA library: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module.  Nothing in ``arborx_gb300`` imports it.

Parity status: pinned by the known-answer vectors of the reference's own tests
(``tests/golden/``) plus exact brute-force cross-checks; the reference itself
cannot be compiled here (Kokkos >= 4.5 is absent).
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libabx_oracle.so")

INTERNAL_DTYPE = np.dtype([("left_child", "<i4"), ("rope", "<i4"), ("box", "<f4", (6,))])
LEAF_DTYPE = np.dtype([("rope", "<i4"), ("value", "<i4")])
assert INTERNAL_DTYPE.itemsize == 32 and LEAF_DTYPE.itemsize == 8

KIND_POINT, KIND_SPHERE, KIND_BOX = 0, 1, 2
MODE_ARBORX, MODE_ORDERED = 0, 1

_lib = None


def build_oracle(verbose=False):
    """Compile the C oracle with its Makefile (gcc, no GPU needed)."""
    cmd = ["make", "-s", "-C", _HERE]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if verbose and out.stdout:
        print(out.stdout)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "abx_oracle.c")
        ):
            build_oracle()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        I32 = ctypes.c_int32
        I = ctypes.c_int
        L.abxo_expand_bits64.restype = ctypes.c_uint64
        L.abxo_expand_bits64.argtypes = [ctypes.c_uint64, I]
        L.abxo_expand_bits32.restype = ctypes.c_uint32
        L.abxo_expand_bits32.argtypes = [ctypes.c_uint32, I]
        L.abxo_morton64.restype = ctypes.c_uint64
        L.abxo_morton64.argtypes = [P, I]
        L.abxo_morton32.restype = ctypes.c_uint32
        L.abxo_morton32.argtypes = [P, I]
        L.abxo_scene_bounds.argtypes = [P, I64, I, P]
        L.abxo_morton64_codes.argtypes = [P, I64, I, P, P]
        L.abxo_morton32_codes.argtypes = [P, I64, I, P, P]
        L.abxo_sort_u64.argtypes = [P, I64, P]
        L.abxo_sort_u32.argtypes = [P, I64, P]
        L.abxo_generate_hierarchy.argtypes = [P, I64, I, P, P, P, P]
        L.abxo_build.argtypes = [P, I64, I, P, P, P, P, P]
        L.abxo_spatial_count.restype = I64
        L.abxo_spatial_count.argtypes = [I64, I, P, P, P, I, P, I64, P]
        L.abxo_spatial_fill.argtypes = [I64, I, P, P, P, I, P, I64, P, P]
        L.abxo_nearest.restype = I64
        L.abxo_nearest.argtypes = [I64, I, P, P, P, P, I64, P, I32, I, P, P, P]
        L.abxo_knn_brute.argtypes = [P, I64, I, P, I64, I32, P, P]
        L.abxo_spatial_brute.restype = I64
        L.abxo_spatial_brute.argtypes = [P, I64, I, I, P, I64, P, P]
        L.abxo_exclusive_scan_i32.argtypes = [P, I64, P]
        for name in ("abxo_kdop_empty",):
            getattr(L, name).argtypes = [I, P]
        L.abxo_kdop_expand_point.argtypes = [I, P, P]
        L.abxo_kdop_expand_box.argtypes = [I, P, P]
        L.abxo_kdop_intersects_kdop.argtypes = [I, P, P]
        L.abxo_kdop_intersects_box.argtypes = [I, P, P]
        L.abxo_point_intersects_kdop.argtypes = [I, P, P]
        L.abxo_kdop_from_geometry.argtypes = [I, I, P, I64, P]
        L.abxo_kdop_axis_boxes.argtypes = [I, P, I64, P]
        L.abxo_kdop_spatial_brute.restype = I64
        L.abxo_kdop_spatial_brute.argtypes = [P, I64, I, I, P, I64, I, I, P, P]
        L.abxo_visit_counts.argtypes = [I64, I, P, P, P, I, I, P, I64, I32, P, P]
        L.abxo_ray_normalize.argtypes = [P, I64, P]
        L.abxo_ray_box_intersection.restype = I
        L.abxo_ray_box_intersection.argtypes = [P, P, P, P]
        L.abxo_ray_box_intersects.restype = I
        L.abxo_ray_box_intersects.argtypes = [P, P]
        L.abxo_ray_box_distance.restype = ctypes.c_float
        L.abxo_ray_box_distance.argtypes = [P, P]
        L.abxo_ray_brute.restype = I64
        L.abxo_ray_brute.argtypes = [P, I64, I, P, I64, I, P, P, P]
        L.abxo_ray_ordered_tree.restype = I64
        L.abxo_ray_ordered_tree.argtypes = [I64, I, P, P, P, P, I64, P, P, P]
        L.abxo_ray_nearest_arborx.restype = I64
        L.abxo_ray_nearest_arborx.argtypes = [I64, I, P, P, P, P, I64, I, P, P, P]
        L.abxo_half_neighbors.restype = I64
        L.abxo_half_neighbors.argtypes = [I64, P, P, P, ctypes.c_float, P, P]
        L.abxo_num_threads.restype = I
        L.abxo_set_num_threads.argtypes = [I]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(a, cols):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.size == 0:
        return a.reshape(0, cols)
    return a.reshape(-1, cols)


def ray_normalize(rays):
    """Ray{origin, direction} construction (ArborX_Ray.hpp:46-55): rows of 6
    floats with the direction normalized as the reference does."""
    r = _f32(rays, 6)
    out = np.empty_like(r)
    lib().abxo_ray_normalize(_p(r), r.shape[0], _p(out))
    return out


def ray_box_intersection(ray, box):
    """(hit, tmin, tmax) of intersection(Ray, Box) (ArborX_Ray.hpp:107-158);
    ray already normalized."""
    r = _f32(ray, 6)
    b = _f32(box, 6)
    t0 = np.zeros(1, np.float32)
    t1 = np.zeros(1, np.float32)
    hit = lib().abxo_ray_box_intersection(_p(r), _p(b), _p(t0), _p(t1))
    return bool(hit), float(t0[0]), float(t1[0])


def ray_box_intersects(ray, box):
    return bool(lib().abxo_ray_box_intersects(_p(_f32(ray, 6)), _p(_f32(box, 6))))


def ray_box_distance(ray, box):
    return lib().abxo_ray_box_distance(_p(_f32(ray, 6)), _p(_f32(box, 6)))


def ray_brute(geom, rays, ordered, is_box=True):
    """CRS (offsets, indices, distances) of intersects(ray) (ascending index)
    or ordered_intersects(ray) (ascending (distance, index)) by brute force;
    rays already normalized."""
    g = _f32(geom, 6 if is_box else 3)
    r = _f32(rays, 6)
    nq = r.shape[0]
    offsets = np.zeros(nq + 1, np.int32)
    total = lib().abxo_ray_brute(_p(g), g.shape[0], int(is_box), _p(r), nq, int(ordered),
                                 _p(offsets), None, None)
    indices = np.empty(total, np.int32)
    dist = np.empty(total, np.float32)
    lib().abxo_ray_brute(_p(g), g.shape[0], int(is_box), _p(r), nq, int(ordered), _p(offsets),
                         _p(indices), _p(dist))
    return offsets, indices, dist


def num_threads():
    return lib().abxo_num_threads()


def set_num_threads(n):
    lib().abxo_set_num_threads(int(n))


def expand_bits64(x, n_zero):
    return int(lib().abxo_expand_bits64(int(x), int(n_zero)))


def expand_bits32(x, n_zero):
    return int(lib().abxo_expand_bits32(int(x), int(n_zero)))


def morton64(p):
    a = np.ascontiguousarray(p, dtype=np.float32).reshape(-1)
    return int(lib().abxo_morton64(_p(a), a.size))


def morton32(p):
    a = np.ascontiguousarray(p, dtype=np.float32).reshape(-1)
    return int(lib().abxo_morton32(_p(a), a.size))


def scene_bounds(geom, is_box=False):
    g = _f32(geom, 6 if is_box else 3)
    out = np.empty(6, np.float32)
    lib().abxo_scene_bounds(_p(g), g.shape[0], int(is_box), _p(out))
    return out


def morton64_codes(geom, scene, is_box=False):
    g = _f32(geom, 6 if is_box else 3)
    s = np.ascontiguousarray(scene, dtype=np.float32)
    out = np.empty(g.shape[0], np.uint64)
    lib().abxo_morton64_codes(_p(g), g.shape[0], int(is_box), _p(s), _p(out))
    return out


def morton32_codes(geom, scene, kind):
    g = _f32(geom, {KIND_POINT: 3, KIND_SPHERE: 4, KIND_BOX: 6}[kind])
    s = np.ascontiguousarray(scene, dtype=np.float32)
    out = np.empty(g.shape[0], np.uint32)
    lib().abxo_morton32_codes(_p(g), g.shape[0], int(kind), _p(s), _p(out))
    return out


def sort_u64(keys):
    k = np.array(keys, dtype=np.uint64, copy=True)
    perm = np.empty(k.size, np.uint32)
    lib().abxo_sort_u64(_p(k), k.size, _p(perm))
    return k, perm


def sort_u32(keys):
    k = np.array(keys, dtype=np.uint32, copy=True)
    perm = np.empty(k.size, np.uint32)
    lib().abxo_sort_u32(_p(k), k.size, _p(perm))
    return k, perm


def generate_hierarchy(geom, perm, sorted_codes, is_box=False):
    g = _f32(geom, 6 if is_box else 3)
    n = g.shape[0]
    perm = np.ascontiguousarray(perm, dtype=np.uint32)
    codes = np.ascontiguousarray(sorted_codes, dtype=np.uint64)
    leaves = np.zeros(n, LEAF_DTYPE)
    internal = np.zeros(max(n - 1, 0), INTERNAL_DTYPE)
    lib().abxo_generate_hierarchy(_p(g), n, int(is_box), _p(perm), _p(codes), _p(leaves), _p(internal))
    return leaves, internal


def exclusive_scan(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    out = np.empty_like(a)
    lib().abxo_exclusive_scan_i32(_p(a), a.size, _p(out))
    return out


class OracleTree:
    """ArborX BVH built on the CPU: tree arrays in the reference layout."""

    def __init__(self, geom, is_box=False):
        self.is_box = bool(is_box)
        self.geom = _f32(geom, 6 if is_box else 3)
        n = self.geom.shape[0]
        self.n = n
        self.bounds = np.empty(6, np.float32)
        self.sorted_codes = np.zeros(n, np.uint64)
        self.perm = np.zeros(n, np.uint32)
        self.leaves = np.zeros(n, LEAF_DTYPE)
        self.internal = np.zeros(max(n - 1, 0), INTERNAL_DTYPE)
        lib().abxo_build(
            _p(self.geom), n, int(self.is_box), _p(self.bounds), _p(self.sorted_codes),
            _p(self.perm), _p(self.leaves), _p(self.internal),
        )

    def _tree_args(self):
        return (self.n, int(self.is_box), _p(self.geom), _p(self.leaves), _p(self.internal))

    def spatial(self, kind, preds):
        """CRS (offsets, indices) of intersects(Sphere|Box) predicates."""
        preds = _f32(preds, 4 if kind == KIND_SPHERE else 6)
        nq = preds.shape[0]
        offsets = np.zeros(nq + 1, np.int32)
        total = lib().abxo_spatial_count(*self._tree_args(), int(kind), _p(preds), nq, _p(offsets))
        indices = np.empty(total, np.int32)
        lib().abxo_spatial_fill(*self._tree_args(), int(kind), _p(preds), nq, _p(offsets), _p(indices))
        return offsets, indices

    def nearest(self, queries, k, mode=MODE_ORDERED):
        """CRS (offsets, indices, distances) of nearest(Point, k) predicates.

        ``k`` is an int or one int per query.  mode MODE_ARBORX restates the
        reference's tie behaviour; MODE_ORDERED keeps the k smallest
        (distance, index) pairs in ascending order (this library's rule).
        """
        q = _f32(queries, 3)
        nq = q.shape[0]
        kq = None
        k_scalar = 0
        if np.ndim(k) == 0:
            k_scalar = int(k)
            total = nq * max(0, min(k_scalar, self.n))
        else:
            kq = np.ascontiguousarray(k, dtype=np.int32)
            total = int(np.minimum(np.maximum(kq, 0), self.n).sum())
        offsets = np.zeros(nq + 1, np.int32)
        indices = np.empty(total, np.int32)
        dist = np.empty(total, np.float32)
        r = lib().abxo_nearest(
            *self._tree_args(), _p(q), nq, _p(kq), k_scalar, int(mode), _p(offsets), _p(indices), _p(dist)
        )
        if r < 0:
            raise RuntimeError("oracle nearest traversal overflowed its 64-entry stack")
        return offsets, indices, dist

    def ray_ordered(self, rays):
        """CRS (offsets, indices, distances) of ordered_intersects(Ray) by the
        reference's best-first traversal restated step for step
        (ArborX_TreeTraversal.hpp:338-489), in its report order; rays
        already normalized."""
        r = _f32(rays, 6)
        nq = r.shape[0]
        offsets = np.zeros(nq + 1, np.int32)
        total = lib().abxo_ray_ordered_tree(*self._tree_args(), _p(r), nq, _p(offsets), None, None)
        indices = np.empty(total, np.int32)
        dist = np.empty(total, np.float32)
        lib().abxo_ray_ordered_tree(*self._tree_args(), _p(r), nq, _p(offsets), _p(indices), _p(dist))
        return offsets, indices, dist

    def half_neighbors(self, radius):
        """CRS (offsets, indices) of findHalfNeighborList over this point
        tree by the reference's HalfTraversal restated (ArborX_HalfTraversal.hpp:
        23-75): row p lists the points within radius whose leaf precedes p's,
        in Morton order."""
        assert not self.is_box
        offsets = np.zeros(self.n + 1, np.int32)
        total = lib().abxo_half_neighbors(self.n, _p(self.geom), _p(self.leaves), _p(self.internal),
                                          float(radius), _p(offsets), None)
        indices = np.empty(total, np.int32)
        lib().abxo_half_neighbors(self.n, _p(self.geom), _p(self.leaves), _p(self.internal),
                                  float(radius), _p(offsets), _p(indices))
        return offsets, indices

    def ray_nearest_arborx(self, rays, k):
        """CRS (offsets, indices, distances) of nearest(Ray, k) by the
        reference's nearest traversal restated (ArborX_TreeTraversal.hpp:
        122-336) with distance(Ray, Box); rays already normalized."""
        r = _f32(rays, 6)
        nq = r.shape[0]
        offsets = np.zeros(nq + 1, np.int32)
        total = lib().abxo_ray_nearest_arborx(*self._tree_args(), _p(r), nq, int(k), _p(offsets),
                                              None, None)
        if total < 0:
            raise RuntimeError("oracle nearest traversal overflowed its 64-entry stack")
        indices = np.empty(total, np.int32)
        dist = np.empty(total, np.float32)
        lib().abxo_ray_nearest_arborx(*self._tree_args(), _p(r), nq, int(k), _p(offsets),
                                      _p(indices), _p(dist))
        return offsets, indices, dist


def visit_counts(tree, mode, preds, k=0, kind=KIND_SPHERE):
    """Mean (internal, leaf) node reads per query of the reference traversal:
    mode 0 = nearest(k) over points [nq,3], mode 1 = spatial (kind)."""
    p = _f32(preds, 3 if mode == 0 else (4 if kind == KIND_SPHERE else 6))
    vi = ctypes.c_int64(0)
    vl = ctypes.c_int64(0)
    lib().abxo_visit_counts(*tree._tree_args(), int(mode), int(kind), _p(p), p.shape[0], int(k),
                            ctypes.byref(vi), ctypes.byref(vl))
    return vi.value / max(p.shape[0], 1), vl.value / max(p.shape[0], 1)


def knn_brute(geom, queries, k, is_box=False):
    g = _f32(geom, 6 if is_box else 3)
    q = _f32(queries, 3)
    kk = max(0, min(int(k), g.shape[0]))
    idx = np.empty((q.shape[0], kk), np.int32)
    dist = np.empty((q.shape[0], kk), np.float32)
    lib().abxo_knn_brute(_p(g), g.shape[0], int(is_box), _p(q), q.shape[0], int(k), _p(idx), _p(dist))
    return idx, dist


def spatial_brute(geom, kind, preds, is_box=False):
    g = _f32(geom, 6 if is_box else 3)
    p = _f32(preds, 4 if kind == KIND_SPHERE else 6)
    nq = p.shape[0]
    offsets = np.zeros(nq + 1, np.int32)
    total = lib().abxo_spatial_brute(_p(g), g.shape[0], int(is_box), int(kind), _p(p), nq, _p(offsets), None)
    indices = np.empty(total, np.int32)
    lib().abxo_spatial_brute(_p(g), g.shape[0], int(is_box), int(kind), _p(p), nq, _p(offsets), _p(indices))
    return offsets, indices


# ---------------------------------------------------------------------------
# KDOP<3, k> (src/geometry/ArborX_KDOP.hpp): ndir = k/2 directions, a KDOP is
# 2 * ndir float32 (min[ndir] then max[ndir]).
# ---------------------------------------------------------------------------

KDOP_NDIR = {6: 3, 14: 7, 18: 9, 26: 13}


def kdop_empty(ndir):
    k = np.empty(2 * ndir, np.float32)
    lib().abxo_kdop_empty(ndir, _p(k))
    return k


def kdop_expand(k, geom):
    """expand(KDOP, Point) for a 3-vector, expand(KDOP, Box) for a 6-vector;
    k is updated in place and returned."""
    ndir = k.size // 2
    g = np.ascontiguousarray(geom, np.float32)
    if g.size == 3:
        lib().abxo_kdop_expand_point(ndir, _p(k), _p(g))
    else:
        lib().abxo_kdop_expand_box(ndir, _p(k), _p(g))
    return k


def kdop_intersects(k, other):
    """intersects(KDOP, Point | Box | KDOP) (symmetric)."""
    ndir = k.size // 2
    o = np.ascontiguousarray(other, np.float32)
    if o.size == 3:
        return bool(lib().abxo_point_intersects_kdop(ndir, _p(o), _p(k)))
    if o.size == 6 and ndir != 3:
        return bool(lib().abxo_kdop_intersects_box(ndir, _p(k), _p(o)))
    return bool(lib().abxo_kdop_intersects_kdop(ndir, _p(k), _p(o)))


def kdop_from_geometry(geom, ndir, is_box=False):
    g = _f32(geom, 6 if is_box else 3)
    out = np.empty((g.shape[0], 2 * ndir), np.float32)
    lib().abxo_kdop_from_geometry(ndir, int(is_box), _p(g), g.shape[0], _p(out))
    return out


def kdop_axis_boxes(kdops):
    k = np.ascontiguousarray(kdops, np.float32)
    ndir = k.shape[1] // 2
    out = np.empty((k.shape[0], 6), np.float32)
    lib().abxo_kdop_axis_boxes(ndir, _p(k), k.shape[0], _p(out))
    return out


def kdop_spatial_brute(values, vkind, preds, pkind):
    """CRS of intersects over every value, ascending values per row.  vkind /
    pkind: "point", "box" or a KDOP k (6, 14, 18, 26)."""
    def code(kind):
        if kind == "point":
            return 0, 0, 3
        if kind == "box":
            return 1, 0, 6
        return 2, KDOP_NDIR[kind], 2 * KDOP_NDIR[kind]
    vk, vn, vs = code(vkind)
    pk, pn, ps = code(pkind)
    v = _f32(values, vs)
    p = _f32(preds, ps)
    nq = p.shape[0]
    offsets = np.zeros(nq + 1, np.int32)
    total = lib().abxo_kdop_spatial_brute(_p(v), v.shape[0], vk, vn, _p(p), nq, pk, pn, _p(offsets), None)
    indices = np.empty(total, np.int32)
    lib().abxo_kdop_spatial_brute(_p(v), v.shape[0], vk, vn, _p(p), nq, pk, pn, _p(offsets), _p(indices))
    return offsets, indices


def in_tree_order(offsets, indices, leaf_values):
    """Each CRS row reordered by the leaves' Morton positions (leaf_values:
    the tree's leaf values in Morton order): the order of a depth-first,
    left-first traversal, whatever its pruning."""
    pos = np.empty(len(leaf_values), np.int64)
    pos[np.asarray(leaf_values)] = np.arange(len(leaf_values))
    out = indices.copy()
    for q in range(len(offsets) - 1):
        a, b = offsets[q], offsets[q + 1]
        row = indices[a:b]
        out[a:b] = row[np.argsort(pos[row], kind="stable")]
    return out


def expand_half_to_full(offsets, indices):
    """ArborX::Details::expandHalfToFull (src/spatial/detail/
    ArborX_ExpandHalfToFull.hpp:23-69): every pair (i, k) of the half list
    counts in rows i and k, an exclusive scan gives the offsets, and the pair
    writes k into row i and i into row k.  Pure Python (small cases); rows in
    insertion order (the reference fills them through atomics, so only their
    contents are defined)."""
    offsets = [int(x) for x in offsets]
    indices = [int(x) for x in indices]
    n = len(offsets) - 1
    counts = [0] * (n + 1)
    for i in range(n):
        for j in range(offsets[i], offsets[i + 1]):
            counts[i] += 1
            counts[indices[j]] += 1
    out_off = [0]
    for i in range(n):
        out_off.append(out_off[-1] + counts[i])
    pos = out_off[:-1]
    out = [0] * out_off[-1]
    for i in range(n):
        for j in range(offsets[i], offsets[i + 1]):
            k = indices[j]
            out[pos[i]] = k
            pos[i] += 1
            out[pos[k]] = i
            pos[k] += 1
    return out_off, out
