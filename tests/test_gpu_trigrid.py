"""The device-built triangle grid of the wall contacts against the numpy
restatement (tests/trigrid_ref.py), bit for bit: dimensions, origin, cell size,
cell starts and the triangle lists in mesh order, for the hopper's cone and
floor (20,002 triangles) and the drum's 65,536 triangles."""
import ctypes
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
from tests import trigrid_ref as tg  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def device_grid(sim):
    L = sim._L
    dims = (ctypes.c_int32 * 3)()
    lc = (ctypes.c_double * 4)()
    ns, ni = ctypes.c_size_t(), ctypes.c_size_t()
    assert L.rp_debug_triangle_grid(sim._h, dims, lc, None, 0, None, 0, ctypes.byref(ns), ctypes.byref(ni)) == 0
    start = np.zeros(ns.value, np.uint32)
    items = np.zeros(max(ni.value, 1), np.uint32)
    u32 = ctypes.POINTER(ctypes.c_uint32)
    assert L.rp_debug_triangle_grid(sim._h, dims, lc, start.ctypes.data_as(u32), ns.value,
                                    items.ctypes.data_as(u32), ni.value, ctypes.byref(ns), ctypes.byref(ni)) == 0
    return tuple(dims), np.array(lc[:3]), lc[3], start, items[:ni.value]


@pytest.mark.parametrize("which", ["hopper", "drum"])
def test_device_grid_matches_restatement(rp, which):
    wl = bench.hopper_workload(n=5000) if which == "hopper" else bench.drum_workload(n=5000)
    sim = bench.make_sim(rp, wl)
    dims, lo, cell, start, items = device_grid(sim)
    rdims, rlo, rcell, rstart, ritems = tg.triangle_grid(wl["tri_v"], float(np.max(wl["radius"])))
    assert dims == rdims
    np.testing.assert_array_equal(lo, rlo)
    assert cell == rcell
    np.testing.assert_array_equal(start, rstart.astype(np.uint32))
    np.testing.assert_array_equal(items, ritems.astype(np.uint32))
    assert len(items) > len(wl["tri_v"])
