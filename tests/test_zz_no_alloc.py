"""The allocation-free cell sort (rp_cell_sort_noalloc) against the
allocating entry point (rp_debug_reference_grid), through the C ABI.

Callers of rp_cell_sort_noalloc cannot allocate device memory themselves in
the code path that calls it (a stream capture in progress, an engine whose pool
owns all device memory, a real-time loop); they hand over their own device
buffers and the library keeps its temporaries in a static device array. The
test owns its buffers (torch tensors), calls the entry point twice in a row
with different inputs, and checks both results bit for bit against the
allocating path on the same positions.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as rp
    from rusty_particles_gb300 import _lib
    return torch, rp, _lib.load()


def allocating_reference(rp, pos, lo, hi, h):
    sim = rp.Simulation.create(1e-4, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], len(pos))
    sim.add_particles(pos, np.full(len(pos), 1e-3), np.full(len(pos), 1.0))
    return sim.debug_reference_grid(h)


def no_alloc(torch, L, pos, lo, dims, h):
    n = len(pos)
    dpos = torch.from_numpy(np.ascontiguousarray(pos, np.float64).reshape(-1)).cuda()
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    origin = (ctypes.c_double * 3)(*lo)
    d = (ctypes.c_int32 * 3)(*dims)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.rp_cell_sort_noalloc(ctypes.cast(dpos.data_ptr(), ctypes.POINTER(ctypes.c_double)), n, origin, h, d,
                                ctypes.c_void_p(cell.data_ptr()), ctypes.c_void_p(order.data_ptr()),
                                ctypes.c_void_p(stream))
    assert rc == 0, L.rp_last_error()
    torch.cuda.synchronize()
    return cell.cpu().numpy().view(np.uint32), order.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("case", [(11, 5000, 0.05), (12, 200_000, 0.01)])
def test_two_calls_match_allocating_path(env, case):
    torch, rp, L = env
    lo, hi = (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)
    results = []
    for call in range(2):  # two calls in a row share the scratch array
        seed, n, h = case
        rng = np.random.default_rng(seed + 100 * call)
        pos = rng.uniform(-0.6, 0.6, (n + 37 * call, 3))  # some particles outside the grid
        dims, cell_ref, order_ref = allocating_reference(rp, pos, lo, hi, h)
        cell, order = no_alloc(torch, L, pos, lo, dims, h)
        inside = cell_ref >= 0
        np.testing.assert_array_equal(cell[inside], cell_ref[inside].astype(np.uint32))
        assert np.all(cell[~inside] == 0xFFFFFFFF)
        k = len(order_ref)
        np.testing.assert_array_equal(order[:k], order_ref.astype(np.uint32))
        np.testing.assert_array_equal(order[k:], np.flatnonzero(~inside).astype(np.uint32))
        results.append(order)
    assert len(results[0]) != len(results[1])


def test_calls_allocate_nothing(env):
    # After one warm-up call (which looks up the scratch array's address), the
    # entry point must not change the device's free memory: every buffer is
    # the caller's, every temporary lives in the static array.
    torch, rp, L = env
    n = 100_000
    rng = np.random.default_rng(5)
    dpos = torch.from_numpy(rng.uniform(-0.5, 0.5, 3 * n)).cuda()
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    origin = (ctypes.c_double * 3)(-0.5, -0.5, -0.5)
    d = (ctypes.c_int32 * 3)(21, 21, 21)
    stream = torch.cuda.current_stream().cuda_stream
    args = (ctypes.cast(dpos.data_ptr(), ctypes.POINTER(ctypes.c_double)), n, origin, 0.05, d,
            ctypes.c_void_p(cell.data_ptr()), ctypes.c_void_p(order.data_ptr()), ctypes.c_void_p(stream))
    assert L.rp_cell_sort_noalloc(*args) == 0, L.rp_last_error()
    torch.cuda.synchronize()
    first = order.cpu().clone()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert L.rp_cell_sort_noalloc(*args) == 0, L.rp_last_error()
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_before - free_after < (1 << 20), (free_before, free_after)
    assert torch.equal(order.cpu(), first)


def test_rejects_oversized_input(env):
    torch, rp, L = env
    origin = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    d = (ctypes.c_int32 * 3)(4, 4, 4)
    rc = L.rp_cell_sort_noalloc(None, (1 << 18) + 1, origin, 1.0, d, None, None, None)
    assert rc == -1
    assert b"at most" in L.rp_last_error()
