"""Shared test helpers: fixture decoding and CRS comparisons."""

import numpy as np

FLT_MAX = np.float32(np.finfo(np.float32).max)
EMPTY_BOX = [FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX]


def box_list(items):
    """Boxes from the golden JSON: 'empty' is the default-constructed box."""
    out = [EMPTY_BOX if (isinstance(b, str) and b == "empty") else b for b in items]
    return np.asarray(out, dtype=np.float32).reshape(-1, 6)


def crs_as_sets(offsets, indices):
    offsets = np.asarray(offsets)
    indices = np.asarray(indices)
    return [sorted(indices[offsets[i]:offsets[i + 1]].tolist()) for i in range(len(offsets) - 1)]


def assert_crs_multiset_equal(off_a, ind_a, off_b, ind_b):
    """Same comparison as the reference's make_compressed_storage check
    (test/boost_ext/CompressedStorageComparison.hpp:21-61): offsets equal,
    indices per query equal as multisets."""
    off_a, off_b = np.asarray(off_a), np.asarray(off_b)
    assert off_a.shape == off_b.shape, (off_a.shape, off_b.shape)
    assert np.array_equal(off_a, off_b)
    assert crs_as_sets(off_a, ind_a) == crs_as_sets(off_b, ind_b)


def manufactured_grid(nx=11, L=100.0, seed=0):
    """Boxes and queries of test/tstQueryTreeManufacturedSolution.cpp:64-269.

    Returns leaves (n x 6 degenerate boxes) and three query sets with their
    expected CRS: (i) the leaves themselves, (ii) boxes spanning the first
    neighbours, (iii) grid-step boxes centred within 0.45 h of a random lattice
    point (drawn here with numpy; the reference uses std::default_random_engine,
    the expected answer is the lattice point by construction either way)."""
    n = nx ** 3
    h = np.float32(L) / np.float32(nx - 1)

    def ind(i, j, k):
        return i + j * nx + k * nx * nx

    leaves = np.zeros((n, 6), np.float32)
    for i in range(nx):
        for j in range(nx):
            for k in range(nx):
                p = [np.float32(i) * h, np.float32(j) * h, np.float32(k) * h]
                leaves[ind(i, j, k)] = p + p
    q1 = leaves.copy()
    exp1 = (np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32))

    q2 = np.zeros((n, 6), np.float32)
    sets = []
    for i in range(nx):
        for j in range(nx):
            for k in range(nx):
                q2[ind(i, j, k)] = [
                    np.float32(i - 1) * h, np.float32(j - 1) * h, np.float32(k - 1) * h,
                    np.float32(i + 1) * h, np.float32(j + 1) * h, np.float32(k + 1) * h,
                ]
    for idx in range(n):
        k, rem = divmod(idx, nx * nx)
        j, i = divmod(rem, nx)
        s = []
        for di in (-1, 0, 1):
            for dj in (-1, 0, 1):
                for dk in (-1, 0, 1):
                    a, b, c = i + di, j + dj, k + dk
                    if 0 <= a < nx and 0 <= b < nx and 0 <= c < nx:
                        s.append(ind(a, b, c))
        sets.append(sorted(s))
    off2 = np.zeros(n + 1, np.int32)
    off2[1:] = np.cumsum([len(s) for s in sets])
    exp2 = (off2, np.concatenate([np.asarray(s, np.int32) for s in sets]))

    rng = np.random.default_rng(seed)
    ijk = rng.integers(0, nx, size=(n, 3))
    shift = rng.uniform(-0.45, 0.45, size=(n, 3)).astype(np.float32)
    c = (ijk.astype(np.float32) + shift) * h
    q3 = np.concatenate([c - h / 2, c + h / 2], axis=1).astype(np.float32)
    exp3 = (np.arange(n + 1, dtype=np.int32),
            np.asarray([ind(*t) for t in ijk.tolist()], np.int32))
    return leaves, [(q1, exp1), (q2, exp2), (q3, exp3)]


def uniform_points(n, seed):
    rng = np.random.default_rng(seed)
    return rng.random((n, 3), dtype=np.float32)


def clouds(sizes, seed):
    """Point clouds of the batched workload's shape: cloud i has a lower
    corner in [0, 100)^3, extents 10^U(-1, 1) per axis and sizes[i] points
    uniform in its box.  Returns (points [N,3] f32, offsets [ntrees+1])."""
    rng = np.random.default_rng(seed)
    sizes = np.asarray(sizes, np.int64)
    corner = rng.uniform(0, 100, (sizes.size, 3)).astype(np.float32)
    extent = (10.0 ** rng.uniform(-1, 1, (sizes.size, 3))).astype(np.float32)
    parts = [corner[i] + extent[i] * rng.random((s, 3), dtype=np.float32)
             for i, s in enumerate(sizes)]
    pts = np.concatenate(parts).astype(np.float32) if parts else np.zeros((0, 3), np.float32)
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return pts, offsets, extent


def cloud_box_queries(pts, offsets, extent, frac=0.02):
    """One axis-aligned box per point, centred on it, full edge frac x its
    cloud's extent per axis."""
    tree = np.repeat(np.arange(offsets.size - 1), np.diff(offsets))
    half = (0.5 * frac * extent[tree]).astype(np.float32)
    return np.concatenate([pts - half, pts + half], axis=1).astype(np.float32)
