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


def test_ray_cpu_leg_checks_rows():
    """The ray case's CPU leg: with rows equal to the oracle's it reports
    bit-exact parity; a row with two entries swapped, or one distance off by
    one ulp, is caught."""
    boxes, rays = bench.make_ray_grid(6, 2)
    nrm = o.ray_normalize(rays)
    ro, ri, rd = o.ray_brute(boxes, nrm, ordered=True)
    uo, ui, _ = o.ray_brute(boxes, nrm, ordered=False)

    def ordered_row(q):
        return ri[ro[q]:ro[q + 1]].copy(), rd[ro[q]:ro[q + 1]].copy()

    def hit_row(q):
        return ui[uo[q]:uo[q + 1]][::-1].copy()  # order inside a row is free

    leg = bench.ray_cpu_leg(boxes, rays, 200, ordered_row, hit_row, checked=64)
    assert leg["parity"]["bit_exact"] and leg["parity"]["rays_checked"] == 64
    assert leg["value"] > 0 and leg["unit"] == "rays/s" and leg["kind"] == "port"
    sampled = np.linspace(0, len(rays) - 1, 64).astype(np.int64)
    bad = int(next(q for q in sampled if ro[q + 1] - ro[q] >= 2))

    def swapped(q):
        i, d = ordered_row(q)
        if q == bad:
            i[[0, 1]] = i[[1, 0]]
        return i, d

    def ulp_off(q):
        i, d = ordered_row(q)
        if q == bad:
            d[-1] = np.nextafter(d[-1], np.float32(np.inf))
        return i, d

    assert not bench.ray_cpu_leg(boxes, rays, 50, swapped, hit_row, checked=64)["parity"]["bit_exact"]
    assert not bench.ray_cpu_leg(boxes, rays, 50, ulp_off, hit_row, checked=64)["parity"]["bit_exact"]
