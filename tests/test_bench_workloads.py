"""The benchmark's workload definitions on CPU: sizes, meshes, bounds and
determinism of the seeded synthetic beds that bench.py times (no GPU)."""
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _unit_normals(n):
    return np.allclose(np.linalg.norm(n.astype(np.float64), axis=1), 1.0, atol=1e-6)


def test_hopper_bed_inside_the_cone():
    wl = bench.hopper_workload(n=20_000)
    x, r = wl["position"], wl["radius"]
    assert len(x) == len(r) == 20_000
    assert r.min() >= 1e-3 and r.max() <= 4e-3
    # 100 x 100 quads of the cone as triangle pairs plus the two floor triangles
    assert len(wl["tri_v"]) == 20_002 and _unit_normals(wl["tri_n"])
    lo, hi = np.asarray(wl["lo"]), np.asarray(wl["hi"])
    assert np.all(x >= lo) and np.all(x <= hi)
    # every site inside the 30-degree frustum above its outlet (y = 0.15, radius 20 mm)
    rho = np.hypot(x[:, 0], x[:, 2])
    assert np.all(rho < 0.02 + (x[:, 1] - 0.15) * math.tan(math.radians(30.0)) + 1e-3)
    assert wl["periodic"] == (True, False, True) and wl["settle"] > 0
    again = bench.hopper_workload(n=20_000)
    np.testing.assert_array_equal(again["position"], x)


def test_adhesive_bed_solid_fraction():
    wl = bench.adhesive_workload(n=4096)
    r = wl["radius"]
    L = wl["hi"][0]
    phi = float((4.0 / 3.0 * np.pi * r ** 3).sum()) / L ** 3
    assert phi == pytest.approx(0.35, rel=1e-9)
    assert r.min() >= 5e-6 and r.max() <= 20e-6 and wl["periodic"] == (True, True, True)
    assert np.all(wl["position"] > 0.0) and np.all(wl["position"] < L)
    assert wl["normal"] == "jkr" and wl["velocity"].shape == (4096, 3)


def test_batched_boxes_and_walls():
    wl = bench.batched_workload(n_boxes=8)
    counts, groups = wl["counts"], wl["groups"]
    assert len(counts) == 8 and counts.min() >= 2000 and counts.max() <= 60000
    assert np.array_equal(np.bincount(groups, minlength=8), counts)
    assert np.array_equal(np.bincount(wl["tri_group"], minlength=8), np.full(8, 12))  # a walled box each
    assert len(wl["group_material"]) == 8 and _unit_normals(wl["tri_n"])
    # boxes do not overlap: each box's particles lie inside its own walls
    for b in range(8):
        xb = wl["position"][groups == b]
        vb = wl["tri_v"][wl["tri_group"] == b].reshape(-1, 3)
        assert np.all(xb >= vb.min(0)) and np.all(xb <= vb.max(0))


def test_drum_mesh():
    v, n = bench.drum_triangles(0.5, 0.3)
    assert len(v) == 65_536 and _unit_normals(n)
    # normals of the cylinder wall point inward (towards the axis)
    c = v.reshape(-1, 3, 3).mean(1)
    wall = np.abs(np.hypot(c[:, 0], c[:, 1]) - 0.5) < 0.01
    assert np.all((n[wall, 0] * c[wall, 0] + n[wall, 1] * c[wall, 1]) < 0.0)


def test_small_drum_fill():
    wl = bench.drum_workload(n=20_000)
    x = wl["position"]
    assert len(x) == 20_000 and np.all(np.hypot(x[:, 0], x[:, 1]) < 0.5)
    assert wl["tri_motion"][1][2] == pytest.approx(np.pi)  # 30 rpm about z
