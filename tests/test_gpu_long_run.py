"""1e5-step statistical agreement with the reference algorithm.

A sheared frictional bed is chaotic: force differences at the rounding level
grow until single trajectories decorrelate, so one GPU run and one oracle run
are two draws of the same dynamics and their time averages differ by the
bed's own fluctuation (2.7 % in kinetic energy for one 500-sphere bed). The
test therefore compares ensembles: every member of the belt-bed ensemble
(tests/belt_ensemble.py) runs as one group of a single GPU simulation, beds
side by side in their own walled boxes, and the means over members of the
time-averaged kinetic energy, coordination number and packing fraction must
agree with the oracle's (tests/golden/belt_ensemble.json, made by
tests/golden/make_belt_ensemble.py) within 0.5 %. Members are paired (same
start on both sides); with 640 members the standard error of the kinetic
energy difference is about 0.15 %. The mixed form (FP32 pair forces, plain
FP64 integrator without the Kahan residuals) is held to the same bar."""
import json
import math
import os

import numpy as np
import pytest

import belt_ensemble as be
import parity_util as pu

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "belt_ensemble.json")
SLOT = 0.08  # box pitch: 60 mm boxes, 20 mm gaps (wider than any cutoff)


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def _ensemble_sim(rp, members, precision=0):
    per = math.ceil(math.sqrt(members))
    offs = [np.array([SLOT * (j % per), 0.0, SLOT * (j // per)]) for j in range(members)]
    parts = [be.member_state(j) for j in range(members)]
    st = {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}
    st["position"] = np.concatenate([p["position"] + o for p, o in zip(parts, offs)])
    lo = be.LO
    hi = (be.LO[0] + SLOT * per, be.HI[1], be.LO[2] + SLOT * math.ceil(members / per))
    g = pu.gpu_sim(rp, st, be.DT, lo, hi, 1, 0, cell=be.CELL, precision=precision)
    g.set_debug(False)
    g.set_particle_groups(np.repeat(np.arange(members, dtype=np.uint32), be.N_PER_BED))
    for j, o in enumerate(offs):
        v, n, floor = be.walls(o)
        g.add_triangles(v[~floor], n[~floor], group=j)
        g.add_triangles(v[floor], n[floor], group=j, motion=be.BELT)
    return g


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_belt_ensemble_statistics_over_1e5_steps(rp, precision):
    if not os.path.exists(GOLDEN):
        pytest.skip("belt ensemble fixture not generated")
    with open(GOLDEN) as f:
        doc = json.load(f)
    members = doc["members"]
    ref = np.array(doc["per_member"])
    g = _ensemble_sim(rp, members, precision)
    n = be.N_PER_BED
    acc, done = np.zeros((members, 3)), 0
    steps = be.sample_steps()
    for s in steps:
        g.steps(s - done)
        done = s
        q = g.get_state()
        assert len(q["radius"]) == members * n
        for j in range(members):
            sl = slice(j * n, (j + 1) * n)
            acc[j] += be.sample(q["position"][sl], q["velocity"][sl], q["angular_velocity"][sl], q["radius"][sl],
                                q["mass"][sl], be.LO[1])
    gpu = acc / len(steps)
    d = gpu - ref
    mean_ref = ref.mean(0)
    rel = d.mean(0) / mean_ref
    sem = d.std(0, ddof=1) / math.sqrt(members) / mean_ref
    print(f"\nmembers {members}: oracle mean {mean_ref}, gpu mean {gpu.mean(0)}, "
          f"(gpu - oracle) / oracle {rel}, standard error {sem}")
    for k, name in enumerate(("kinetic energy", "coordination", "packing")):
        assert abs(rel[k]) <= 0.005, (name, rel[k], sem[k])
