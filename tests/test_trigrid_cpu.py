"""The triangle grid's covering property, on CPU with the numpy restatement:
every triangle within the largest radius of a point is listed in the cell of
that point (so the wall loop over the cell's triangles finds every contact of
the reference's every-triangle loop, src/simulation.rs:464-523), in mesh order."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
from tests import trigrid_ref as tg  # noqa: E402


def _check_covering(tri_v, rmax, points):
    dims, lo, cell, start, items = tg.triangle_grid(tri_v, rmax)
    v = tri_v.astype(np.float64).reshape(-1, 3, 3)
    T = len(v)
    q = np.floor((points - lo) / cell).astype(np.int64)
    inside = np.all((q >= 0) & (q < np.asarray(dims)), axis=1)
    for p, qq, ins in zip(points, q, inside):
        d2 = tg.point_triangle_dist2(np.repeat(p[None], T, 0), v[:, 0], v[:, 1], v[:, 2])
        near = np.flatnonzero(d2 < rmax * rmax)
        if not ins:
            assert len(near) == 0
            continue
        c = qq[0] + dims[0] * (qq[1] + dims[1] * qq[2])
        lst = items[start[c]:start[c + 1]]
        assert np.all(np.diff(lst) > 0)  # mesh order
        assert set(near.tolist()) <= set(lst.tolist())


def test_cone_and_floor_covering():
    wl = bench.hopper_workload(n=2000)
    rng = np.random.default_rng(1)
    tv = wl["tri_v"]
    rmax = float(wl["radius"].max())
    # points near random triangles (within 2 rmax) and anywhere in the box
    v = tv.astype(np.float64).reshape(-1, 3, 3)
    pick = rng.integers(0, len(v), 300)
    bary = rng.dirichlet([1, 1, 1], 300)
    near = np.einsum("ij,ijk->ik", bary, v[pick]) + rng.normal(0, rmax, (300, 3))
    anywhere = rng.uniform(np.asarray(wl["lo"]), np.asarray(wl["hi"]), (100, 3))
    _check_covering(tv, rmax, np.concatenate([near, anywhere]))


def test_degenerate_triangles_keep_their_box():
    tv = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0], [0, 0, 0, 0, 0, 0, 0, 0, 0], [0, 0, 0, 1, 1, 1, 2, 2, 2]], np.float32)
    dims, lo, cell, start, items = tg.triangle_grid(tv, 0.05)
    # the point and the segment are flat: listed in every cell of their grown box
    assert np.count_nonzero(items == 1) >= 1 and np.count_nonzero(items == 2) >= np.prod(dims) // 10
    _check_covering(tv, 0.05, np.random.default_rng(2).uniform(-0.1, 2.1, (200, 3)))


def _wall_far(p, dims, lo, cell, start):
    """The filter's far-from-walls test (wall_far in csrc/k_step.cu) without its
    periodic-face part: the 27 cells around p's cell list no triangle."""
    q = np.floor((p - lo) / cell).astype(np.int64)
    if np.any(q + 1 < 0) or np.any(q - 1 >= np.asarray(dims)):
        return True
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                c = q + np.array([dx, dy, dz])
                if np.any(c < 0) or np.any(c >= np.asarray(dims)):
                    continue
                i = c[0] + dims[0] * (c[1] + dims[1] * c[2])
                if start[i + 1] > start[i]:
                    return False
    return True


def test_far_from_walls_stays_far_within_half_the_skin():
    # a particle flagged far from every triangle at a list rebuild moves less
    # than half the skin (less than a cell) before the next: no triangle can
    # come within the largest radius of it meanwhile. Points just outside the
    # reach of a triangle, moved towards it and at random.
    wl = bench.hopper_workload(n=2000)
    tv = wl["tri_v"]
    rmax = float(wl["radius"].max())
    half_skin = 0.5 * float(wl.get("skin") or 0.2 * rmax)
    dims, lo, cell, start, items = tg.triangle_grid(tv, rmax)
    assert half_skin * 1.01 < cell
    v = tv.astype(np.float64).reshape(-1, 3, 3)
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    rng = np.random.default_rng(5)
    m = 600
    pick = rng.integers(0, len(v), m)
    bary = rng.dirichlet([1, 1, 1], m)
    sign = rng.choice([-1.0, 1.0], m)
    off = rmax + rng.uniform(0.0, 3.0 * cell, m)
    pts = np.einsum("ij,ijk->ik", bary, v[pick]) + (sign * off)[:, None] * nrm[pick]
    far = 0
    for p, t_, s_ in zip(pts, pick, sign):
        if not _wall_far(p, dims, lo, cell, start):
            continue
        far += 1
        d = rng.normal(0, 1, (5, 3))
        d *= (half_skin * rng.uniform(0, 1, 5) / np.linalg.norm(d, axis=1))[:, None]
        d = np.concatenate([d, -s_ * half_skin * nrm[t_][None]])  # straight towards the triangle
        for q in p + d:
            d2 = tg.point_triangle_dist2(np.repeat(q[None], len(v), 0), v[:, 0], v[:, 1], v[:, 2])
            assert float(d2.min()) >= rmax * rmax
    assert far > 50
