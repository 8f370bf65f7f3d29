"""The oracle's benchmark-side variants against its literal form, on CPU.

The reference's CPU step is timed at benchmark sizes with two changes that
keep its arithmetic: the reference grid's cell set to the largest cutoff
instead of 1 m (src/simulation.rs:64-66), and the every-triangle wall loop
(src/simulation.rs:464-523) culled by a triangle grid. The cull keeps the same
contacts in the same order, so results are bit-identical; the smaller cell
finds the same pairs wherever no periodic axis is involved (it only changes
the order of each particle's sum).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _hopper_oracle(oracle_mod, wl, cull, cell=1.0, bulk=True):
    lo, hi = wl["lo"], wl["hi"]
    o = oracle_mod.OracleSimulation(wl["dt"], lo, hi, prec=64)
    o.set_mode(0)
    o.set_cell_size(cell)
    o.set_options(record_pairs=False, keep_contact_map=True)
    o.set_particle_material(*wl["material"])
    o.set_contact_models(wl["normal"], wl["tangential"])
    o.set_periodic_boundary(*wl["periodic"])
    if bulk:
        o.add_particles(wl["position"], wl["radius"], wl["mass"])
    else:
        for p, r, m in zip(wl["position"], wl["radius"], wl["mass"]):
            o.add_particle(p[0], p[1], p[2], r, m)
    o.add_triangles(wl["tri_v"].astype(np.float64), wl["tri_n"].astype(np.float64))
    o.set_wall_cull(cull)
    return o


def test_wall_cull_is_bit_identical(oracle_mod):
    # a 3,000-sphere hopper bed against its 20,002 triangles: the start state
    # overlaps the cone wall and the floor, so many wall contacts exist
    wl = bench.hopper_workload(n=3000)
    wl["position"][:, 1] -= wl["position"][:, 1].min() - 1e-3  # the lowest spheres touch the floor
    a = _hopper_oracle(oracle_mod, wl, cull=False, bulk=False)
    b = _hopper_oracle(oracle_mod, wl, cull=True)
    for _ in range(3):
        a.step()
        b.step()
        Fa, Ta = a.last_forces()
        Fb, Tb = b.last_forces()
        np.testing.assert_array_equal(Fa, Fb)
        np.testing.assert_array_equal(Ta, Tb)
    sa, sb = a.state(), b.state()
    for k in ("x", "v", "w"):
        np.testing.assert_array_equal(sa[k], sb[k])


def test_cutoff_cell_same_pairs_without_periodic_axes(oracle_mod):
    from tests import parity_util as pu
    lo, hi = (-0.25, -0.25, -0.25), (0.25, 0.25, 0.25)
    st = pu.random_bed(21, 2000, lo, hi, 0.008, 0.012)
    a = pu.oracle_sim(oracle_mod, st, 1e-5, lo, hi, 1, 2, cell=1.0)
    b = pu.oracle_sim(oracle_mod, st, 1e-5, lo, hi, 1, 2, cell=0.024)
    a.step()
    b.step()
    assert pu.pair_counter_oracle(a) == pu.pair_counter_oracle(b)
    Fa, _ = a.last_forces()
    Fb, _ = b.last_forces()
    FS, _ = a.last_force_scale()
    err = np.linalg.norm(Fa - Fb, axis=1) / np.maximum(FS, 1e-300)
    assert float(err.max()) <= 1e-12
