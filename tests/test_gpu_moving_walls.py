"""Moving walls (an extension: the reference's walls are static): triangles
whose surface moves with V + W x (p - C) enter the wall contact's relative
velocity at the contact point (src/simulation.rs:464-523 otherwise unchanged).
The oracle implements the same rule; one step from the same state must agree
as every other wall contact does, and a belt must drag the bed along."""
import numpy as np
import pytest

import parity_util as pu
from stl_util import floor_tris

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def _tris(tris):
    v = np.array([np.concatenate(t) for t in tris], np.float32)
    n = np.array([np.cross(t[1] - t[0], t[2] - t[0]) / np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0]))
                  for t in tris], np.float32)
    return v, n


def _bed():
    lo, hi = (-0.2, 0.0, -0.2), (0.2, 0.4, 0.2)
    st = pu.random_bed(21, 1500, (-0.15, 0.0, -0.15), (0.15, 0.1, 0.15), 0.008, 0.012, vscale=0.02,
                       ascale=0.0, tscale=0.0)
    st["position"][:, 1] += 0.011 - st["position"][:, 1].min()  # lowest layer touches the floor
    return st, lo, hi


@pytest.mark.parametrize("normal", [1, 0, 4])
def test_moving_walls_match_oracle(rp, oracle_mod, normal):
    st, lo, hi = _bed()
    floor = _tris([(np.array(t[0], float), np.array(t[1], float), np.array(t[2], float)) for t in floor_tris()])
    # a belt floor and a plane turning about the y axis through the bed
    belt = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.3, 0.0, 0.05))
    tilt = _tris([(np.array([-0.2, 0.0, 0.13]), np.array([0.2, 0.0, 0.13]), np.array([0.2, 0.4, 0.14])),
                  (np.array([-0.2, 0.0, 0.13]), np.array([0.2, 0.4, 0.14]), np.array([-0.2, 0.4, 0.14]))])
    spin = ((0.0, 0.1, 0.0), (0.0, 2.0, 0.0), (0.0, 0.0, 0.0))
    mat = (1e7, 0.3, 2500.0, 0.5, 0.5, 0.05 if normal == 4 else 0.0)
    o = pu.oracle_sim(oracle_mod, st, 1e-5, lo, hi, normal, 0, material=mat)
    o.add_triangles(floor[0], floor[1], motion=belt)
    o.add_triangles(tilt[0], tilt[1], motion=spin)
    g = pu.gpu_sim(rp, st, 1e-5, lo, hi, normal, 0, material=mat)
    g.add_triangles(floor[0], floor[1], motion=belt)
    g.add_triangles(tilt[0], tilt[1], motion=spin)
    o.step()
    g.step()
    so, sg = o.state(), g.get_state()
    np.testing.assert_array_equal(sg["position"], so["x"])
    Fo, To = o.last_forces()
    Fg, Tg = g.debug_forces()
    FS, TS = o.last_force_scale()
    m = FS > 0
    assert m.sum() > 100
    ef = np.linalg.norm(Fg - Fo, axis=1)[m] / FS[m]
    et = np.linalg.norm(Tg - To, axis=1)[m] / TS[m]
    assert float(ef.max()) <= 1e-9 and float(et.max()) <= 1e-9


def test_belt_drags_the_bed(rp):
    st, lo, hi = _bed()
    floor = _tris([(np.array(t[0], float), np.array(t[1], float), np.array(t[2], float)) for t in floor_tris()])
    g = pu.gpu_sim(rp, st, 1e-5, lo, hi, 1, 0)
    g.set_debug(False)
    g.add_triangles(floor[0], floor[1], motion=((0, 0, 0), (0, 0, 0), (0.5, 0.0, 0.0)))
    low = st["position"][:, 1] < 0.02
    g.steps(2000)
    v = g.get_state()["velocity"]
    # friction on the belt (mu g ~ 4.9 m/s^2 on the lowest layer) accelerates it along +x for 20 ms
    assert v[low, 0].mean() > 0.02
    assert abs(v[low, 2].mean()) < 0.5 * v[low, 0].mean()
