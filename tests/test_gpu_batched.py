"""Groups: independent beds stepped in one simulation.

Each group must behave exactly as its own reference simulation: a batched GPU
run of several walled boxes (different sizes, per-box surface energy, sJKR +
Coulomb, one call stepping all of them) is compared box by box with one
oracle simulation per box (the reference algorithm, src/simulation.rs:156-562)
from the same state: positions bit-exact, per-particle forces within 1e-9 of
the sum of contact-force magnitudes, the contact multiset identical."""
import numpy as np
import pytest

import parity_util as pu
from stl_util import box_tris

pytestmark = pytest.mark.gpu

DT = 1e-6
LO, HI = (0.0, 0.0, 0.0), (0.4, 0.1, 0.1)


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def _boxes(seed, count):
    """count boxes along x with 2 mm gaps, sides 12-30 mm, radii U[0.5, 1.5] mm,
    a touching jittered bed in each, per-box surface energy U[0, 0.1]."""
    rng = np.random.default_rng(seed)
    out = []
    x0 = 0.005
    for b in range(count):
        side = float(rng.uniform(0.012, 0.03))
        lo = np.array([x0, 0.005, 0.005])
        hi = lo + side
        x0 = hi[0] + 0.01
        st = pu.random_bed(seed * 100 + b, 100000, lo + 0.0015, hi - 0.0015, 0.0005, 0.0015, vscale=0.05,
                           ascale=0.0, tscale=0.0)
        st["mass"] = 2500.0 * 4.0 / 3.0 * np.pi * st["radius"] ** 3
        tris = box_tris(lo, hi)
        v = np.array([np.concatenate(t) for t in tris], np.float32)
        n = np.array([np.cross(t[1] - t[0], t[2] - t[0]) / np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0]))
                      for t in tris], np.float32)
        gamma = float(rng.uniform(0.0, 0.1))
        out.append({"st": st, "tri": (v, n), "mat": (1e7, 0.3, 2500.0, 0.5, 0.5, gamma)})
    return out


def _batched_sim(rp, boxes, normal, tangential):
    allst = {k: np.concatenate([b["st"][k] for b in boxes]) for k in boxes[0]["st"]}
    s = rp.Simulation.create(DT, *LO, *HI, len(allst["radius"]))
    s.set_particle_material(*boxes[0]["mat"])
    s.set_contact_models(pu.NORMAL_NAMES[normal], pu.TANGENTIAL_NAMES[tangential])
    s.add_particles(allst["position"], allst["radius"], allst["mass"], allst["fixed"])
    groups = np.concatenate([np.full(len(b["st"]["radius"]), g, np.uint32) for g, b in enumerate(boxes)])
    s.set_particle_groups(groups)
    for g, b in enumerate(boxes):
        if g:
            s.set_group_material(g, *b["mat"])
        s.add_triangles(b["tri"][0], b["tri"][1], group=g)
    s.set_state({k: allst[k] for k in ("velocity", "angular_velocity", "acceleration", "torque")})
    s.set_debug(True)
    return s, groups


@pytest.mark.parametrize("normal,tangential", [(4, 0), (1, 0), (3, 0)])
def test_batched_boxes_match_separate_reference_runs(rp, oracle_mod, normal, tangential):
    boxes = _boxes(3, 5)
    g, groups = _batched_sim(rp, boxes, normal, tangential)
    assert np.array_equal(g.get_particle_groups(), groups)
    oracles = [pu.oracle_sim(oracle_mod, b["st"], DT, LO, HI, normal, tangential, material=b["mat"], tris=b["tri"])
               for b in boxes]
    for steps in (1, 3):
        g.steps(steps)
        for o in oracles:
            o.steps(steps)
        sg = g.get_state()
        Fg, Tg = g.debug_forces()
        pi, pj, vv = g.debug_pairs()
        off = 0
        for b, o in zip(boxes, oracles):
            n = len(b["st"]["radius"])
            so = o.state()
            sl = slice(off, off + n)
            if steps == 1:
                np.testing.assert_array_equal(sg["position"][sl], so["x"])
            else:
                # forces agree to 1e-9, not bit for bit: later positions to rounding
                assert np.max(np.abs(sg["position"][sl] - so["x"])) <= 1e-15
                assert np.max(np.abs(sg["velocity"][sl] - so["v"])) <= 1e-9 * max(1.0, np.abs(so["v"]).max())
            Fo, To = o.last_forces()
            FS, TS = o.last_force_scale()
            m = FS > 0
            ef = np.linalg.norm(Fg[sl] - Fo, axis=1)[m] / FS[m]
            et = np.linalg.norm(Tg[sl] - To, axis=1)[m] / TS[m]
            assert float(ef.max(initial=0)) <= 1e-9 and float(et.max(initial=0)) <= 1e-9
            # contacts of this box only, as the box's own run sees them
            mine = (pi >= off) & (pi < off + n)
            assert np.all((pj[mine] >= off) & (pj[mine] < off + n))
            from collections import Counter
            cg = Counter()
            for a, c, v in zip(pi[mine] - off, pj[mine] - off, vv[mine]):
                cg[(int(a), int(c))] += int(v)
            assert cg == pu.pair_counter_oracle(o)
            off += n


def test_groups_are_independent_when_overlapping_in_space(rp):
    # two identical beds at the same place in two groups: each evolves as if
    # alone (no cross-group contacts), so both stay identical
    lo, hi = (0.0, 0.0, 0.0), (0.02, 0.02, 0.02)
    st = pu.random_bed(9, 300, lo, hi, 0.0005, 0.0015, ascale=0.0, tscale=0.0)
    st["mass"] = 2500.0 * 4.0 / 3.0 * np.pi * st["radius"] ** 3
    n = len(st["radius"])
    s = rp.Simulation.create(DT, -0.1, -0.1, -0.1, 0.1, 0.1, 0.1, 2 * n)
    s.set_contact_models("hertz", "coulomb")
    s.add_particles(np.concatenate([st["position"]] * 2), np.concatenate([st["radius"]] * 2),
                    np.concatenate([st["mass"]] * 2))
    s.set_particle_groups(np.repeat(np.array([0, 1], np.uint32), n))
    s.set_state({"velocity": np.concatenate([st["velocity"]] * 2)})
    s.steps(20)
    out = s.get_state()
    np.testing.assert_array_equal(out["position"][:n], out["position"][n:])
    np.testing.assert_array_equal(out["velocity"][:n], out["velocity"][n:])
