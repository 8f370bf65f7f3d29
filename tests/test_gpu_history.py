"""Tangential spring history across Verlet-list rebuilds (physical mode).

The reference keeps one spring per contact in a map that outlives every step
(src/contact.rs:4-17, src/simulation.rs:397-399); the oracle keys it by the
pair's stable tags. The GPU stores the spring of each directed pair in its
Verlet-row entry and carries it to the new row when the lists are rebuilt
(the pair is looked up in the old row through the reorder permutation). Here
a sheared bed with a Verlet skin of a few step displacements rebuilds its
lists every step or two while the springs are loaded, and every step is
compared with the oracle: positions to 1e-12 m, forces and torques to 1e-9 of
each particle's sum of contact-force magnitudes.
"""
import numpy as np
import pytest

from tests import parity_util as pu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def sheared_bed(seed, n, lo, hi):
    st = pu.random_bed(seed, n, lo, hi, 0.008, 0.012, vscale=0.02, wscale=0.5, ascale=0.0, tscale=0.0)
    y = st["position"][:, 1]
    st["velocity"][:, 0] += 4.0 * (y - y.mean())  # simple shear, |v_x| up to ~1 m/s
    return st


@pytest.mark.parametrize("tangential", [2, 1], ids=["mindlin", "linear_spring"])
def test_springs_survive_rebuilds(rp, oracle_mod, tangential):
    lo, hi = (-0.25, -0.25, -0.25), (0.25, 0.25, 0.25)
    st = sheared_bed(61 + tangential, 2000, lo, hi)
    dt = 1e-5
    o = pu.oracle_sim(oracle_mod, st, dt, lo, hi, 1, tangential, mode=1)
    g = pu.gpu_sim(rp, st, dt, lo, hi, 1, tangential, mode=1)
    g.set_skin(3e-5)  # a particle at 1 m/s crosses half of it in 1.5 steps
    r0 = g.stats()["neighbor_rebuilds"]
    worst_f = worst_x = 0.0
    loaded = 0
    for step in range(60):
        o.step()
        g.step()
        so, sg = o.state(), g.get_state()
        dx = float(np.max(np.abs(sg["position"] - so["x"])))
        assert dx <= 1e-12, (step, dx)
        Fo, To = o.last_forces()
        Fg, Tg = g.debug_forces()
        FS, TS = o.last_force_scale()
        m = FS > 0
        ef = np.linalg.norm(Fg - Fo, axis=1)[m] / FS[m]
        et = np.linalg.norm(Tg - To, axis=1)[m] / TS[m]
        assert float(ef.max(initial=0)) <= 1e-9, (step, float(ef.max()))
        assert float(et.max(initial=0)) <= 1e-9, (step, float(et.max()))
        worst_f = max(worst_f, float(ef.max(initial=0)))
        worst_x = max(worst_x, dx)
        # the springs carry load: torques (r_a x f, only tangential forces
        # make them) on most particles in contact
        loaded = max(loaded, int(np.count_nonzero(np.linalg.norm(To, axis=1) > 1e-6 * TS)))
    rebuilds = g.stats()["neighbor_rebuilds"] - r0
    assert rebuilds >= 20, rebuilds
    assert loaded > 500, loaded
    print(f"\n{rebuilds} rebuilds in 60 steps, worst force error {worst_f:.2e}, worst position error {worst_x:.2e}")

