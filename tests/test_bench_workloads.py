"""The synthetic workloads of bench.py on the host: the raytracing example's
scene (examples/raytracing/example_raytracing.cpp:218-280) and its
properties under the oracle's ray restatement."""

import numpy as np

import bench
from oracle import oracle as o


def test_ray_grid_layout():
    nx, per = 6, 3
    boxes, rays = bench.make_ray_grid(nx, per)
    d = np.float32(100.0 / nx)
    assert boxes.shape == (nx ** 3, 6) and rays.shape == (nx ** 3 * per, 6)
    assert boxes.dtype == np.float32 and rays.dtype == np.float32
    for cid in (0, 1, nx, nx * nx, nx ** 3 - 1):
        i, j, k = cid % nx, (cid // nx) % nx, cid // (nx * nx)
        want = np.array([i, j, k, i + 1, j + 1, k + 1], np.float32) * d
        assert np.array_equal(boxes[cid], want)
    cell = np.repeat(np.arange(nx ** 3), per)
    assert np.all(rays[:, :3] >= boxes[cell, :3]) and np.all(rays[:, :3] <= boxes[cell, 3:])
    assert np.allclose(np.linalg.norm(rays[:, 3:].astype(np.float64), axis=1), 1.0, atol=1e-6)


def test_ray_grid_first_hit_is_the_origin_cell():
    """A ray starting strictly inside its cell enters it at distance 0, and no
    other cell contains the origin, so the cell leads its ordered row."""
    nx, per = 8, 2
    boxes, rays = bench.make_ray_grid(nx, per)
    inside = np.all((rays[:, :3] > np.repeat(boxes[:, :3], per, 0))
                    & (rays[:, :3] < np.repeat(boxes[:, 3:], per, 0)), axis=1)
    sample = np.flatnonzero(inside)[:200]
    off, ind, dist = o.ray_brute(boxes, o.ray_normalize(rays[sample]), ordered=True)
    for j, r in enumerate(sample.tolist()):
        assert off[j + 1] > off[j]
        assert ind[off[j]] == r // per and dist[off[j]] == 0.0
        assert np.all(np.diff(dist[off[j]:off[j + 1]]) >= 0)
