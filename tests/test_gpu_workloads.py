"""Parity on scaled-down slices of the benchmark workloads.

Each slice keeps its workload's radii distribution, laws, mesh, periodicity
and material, at a size the oracle steps in seconds: the lognormal hopper bed
in its 20,000-triangle cone (parity and physical Mindlin), the adhesive JKR
gas at solid fraction 0.35 with sigma = 0.05 m/s velocities under every JKR
solver in FP64 and mixed precision, eight batched sJKR boxes with log-uniform
counts, and a drum inside the rotating 65,536-triangle wall. The bed is
relaxed and settled on the GPU, then both sides step from the same state.
Bars: positions bit-exact (FP64 form), contact pairs bit-exact, per-particle
force and torque within 1e-9 of sum_j |f_ij| (FP64), 1e-6 (certified and
learned JKR) or 1e-5 (mixed).
"""
import os
import sys

import numpy as np
import pytest

from tests import parity_util as pu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def settle(rp, wl, steps, mode="parity", jkr=None):
    bench.relax(rp, wl)
    s = bench.make_sim(rp, wl, mode)
    bench.setup_jkr(s, jkr)
    s.steps(steps)
    st = s.get_state()
    del s
    return st


def one_step(rp, oracle_mod, wl, st, mode="parity", precision="fp64", jkr=None, cell=1.0, cull=False, idx=None,
             material=None, tri_sel=None, gpu=None):
    m = 0 if mode == "parity" else 1
    o = bench.oracle_for(wl, st, cell=cell, cull=cull, mode=m, idx=idx, material=material, tri_sel=tri_sel)
    o.set_options(record_pairs=True, keep_contact_map=True)
    o.step()
    if gpu is None:
        g = bench.make_sim(rp, bench.wl_at(wl, st), mode, precision)
        g.set_reference_cell_size(cell)
        bench.setup_jkr(g, jkr)
        bench.set_dynamic_state(g, st)
        g.set_debug(True)
        g.step()
    else:
        g = gpu
    return o, g


def check(o, g, tol, exact_positions=True, idx=None, check_pairs=True):
    so = o.state()
    sg = g.get_state()
    xg = sg["position"] if idx is None else sg["position"][idx]
    if exact_positions:
        np.testing.assert_array_equal(xg, so["x"])
    else:  # after several steps: forces differ at rounding, positions by far less than 1e-12 m
        assert float(np.max(np.abs(xg - so["x"]))) < 1e-12
    if check_pairs and idx is None:
        assert pu.pair_counter_gpu(g) == pu.pair_counter_oracle(o)
    Fo, To = o.last_forces()
    Fg, Tg = g.debug_forces()
    if idx is not None:
        Fg, Tg = Fg[idx], Tg[idx]
    FS, TS = o.last_force_scale()
    r = bench.compare_forces(Fg, Tg, Fo, To, FS, TS)
    assert r["nonfinite_mismatch"] == 0
    assert r["force_rel_sum"] <= tol and r["torque_rel_sum"] <= tol, r
    assert r["force_abs_where_zero_scale"] == 0.0 and r["torque_abs_where_zero_scale"] == 0.0, r
    return r


@pytest.fixture(scope="module")
def hopper(rp):
    wl = bench.hopper_workload(n=20_000)
    return wl, settle(rp, wl, 400)


def test_hopper_slice_parity(rp, oracle_mod, hopper):
    # the reference's own 1 m grid and every-triangle wall loop
    wl, st = hopper
    o, g = one_step(rp, oracle_mod, wl, st)
    r = check(o, g, 1e-9)
    assert r["particles"] == 20_000 and r["force_net_counted"] > 1000


def test_hopper_slice_physical_mindlin(rp, oracle_mod, hopper):
    # springs start from zero on both sides, then 5 steps side by side
    wl, st = hopper
    hc = bench.max_cutoff(wl)
    g = bench.make_sim(rp, bench.wl_at(wl, st), "physical", "fp64")
    bench.set_dynamic_state(g, st)
    g.set_debug(True)
    o = bench.oracle_for(wl, st, cell=hc, cull=True, mode=1)
    o.set_options(record_pairs=True, keep_contact_map=True)
    for k in range(5):
        o.step()
        g.step()
        check(o, g, 1e-9, exact_positions=k == 0)


@pytest.fixture(scope="module")
def adhesive(rp):
    wl = bench.adhesive_workload(n=20_000)
    st = settle(rp, wl, 200, jkr={"solver": "certified"})
    s = bench.make_sim(rp, bench.wl_at(wl, st))
    s.train_jkr_network(samples=1 << 18, epochs=16, seed=3)
    net = s.get_jkr_network()
    del s
    return wl, st, net


@pytest.mark.parametrize("solver,precision,tol", [("newton", "fp64", 1e-9), ("certified", "fp64", 1e-6),
                                                  ("learned", "fp64", 1e-6), ("newton", "mixed", 1e-5),
                                                  ("certified", "mixed", 1e-5), ("learned", "mixed", 1e-5)])
def test_adhesive_slice(rp, oracle_mod, adhesive, solver, precision, tol):
    wl, st, net = adhesive
    assert np.all(np.std(st["velocity"], axis=0) > 0.01)  # a gas, not a settled bed
    o, g = one_step(rp, oracle_mod, wl, st, precision=precision, jkr={"solver": solver, "network": net},
                    cell=bench.max_cutoff(wl), cull=True)
    # the mixed form's integrator does not carry the Kahan residuals of the
    # settled state: its positions differ from the oracle's in the last bits
    check(o, g, tol, exact_positions=precision == "fp64")
    if solver != "newton":
        c = g.jkr_counters()
        assert c["accepted"] > 0 and c["zero"] > 0, c


def test_batched_slice_eight_boxes(rp, oracle_mod):
    wl = bench.batched_workload(n_boxes=8, n_hi=12_000)
    st = settle(rp, wl, 300)
    hc = bench.max_cutoff(wl)
    g = bench.make_sim(rp, bench.wl_at(wl, st))
    g.set_reference_cell_size(hc)
    bench.set_dynamic_state(g, st)
    g.set_debug(True)
    g.step()
    for b in range(8):
        idx = np.flatnonzero(wl["groups"] == b)
        o, _ = one_step(rp, oracle_mod, wl, st, cell=hc, cull=True, idx=idx, material=wl["group_material"][b],
                        tri_sel=wl["tri_group"] == b, gpu=g)
        check(o, g, 1e-9, idx=idx, check_pairs=False)


def test_drum_slice_rotating_wall(rp, oracle_mod):
    wl = bench.drum_workload(n=20_000)
    st = settle(rp, wl, 300)
    o, g = one_step(rp, oracle_mod, wl, st, cell=bench.max_cutoff(wl), cull=True)
    check(o, g, 1e-9)
    # the wall moves: particles touching it are dragged along its surface
    assert len(bench.drum_triangles(0.5, 0.3)[0]) == len(wl["tri_v"]) == 65_536
