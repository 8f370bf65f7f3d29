"""An ensemble of belt-driven beds for long-run statistics.

Each member is 500 spheres (radii U[2.5, 3] mm, E = 1e7 Pa, nu = 0.3,
rho = 2500, e = 0.5, mu = 0.5) in a 60 x 200 x 60 mm walled box whose floor
moves as a belt at 0.3 m/s along x (a surface velocity; the floor itself stays
put), Hertz + Coulomb, dt = 5e-5 s, reference grid cell 10 mm. Members differ
by the seed of their start (a jittered lattice with random velocities). After
2e4 steps the bed is in a sheared steady state; the statistics are averaged
over one sample every 1000 steps up to 1e5 steps.

The statistics, identical for both arms:
* kinetic energy, translational plus rotational (I = 2/5 m r^2);
* coordination number, 2 x (overlapping sphere pairs) / N;
* packing fraction, sphere volume over floor area x (95th percentile of the
  sphere tops - floor)."""
import numpy as np

from parity_util import random_bed
from stl_util import box_tris

N_PER_BED = 500
LO, HI = (-0.03, -0.1, -0.03), (0.03, 0.1, 0.03)
FILL_HI = (0.03, 0.02, 0.03)
RMIN, RMAX = 0.0025, 0.003
DT, CELL = 5e-5, 0.01
BELT = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.3, 0.0, 0.0))  # (centre, omega, velocity)
STEPS, START, EVERY = 100_000, 20_000, 1_000
SEED0 = 5000
AREA = (HI[0] - LO[0]) * (HI[2] - LO[2])


def member_state(j):
    return random_bed(SEED0 + j, N_PER_BED, LO, FILL_HI, RMIN, RMAX, vscale=0.2, ascale=0.0)


def walls(offset=(0.0, 0.0, 0.0)):
    """Box triangles (n x 9), unit normals, and which of them form the floor."""
    off = np.asarray(offset, float)
    tris = box_tris(np.asarray(LO) + off, np.asarray(HI) + off)
    v = np.array([np.concatenate(t) for t in tris], np.float64)
    nrm = np.array([np.cross(t[1] - t[0], t[2] - t[0]) / np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0]))
                    for t in tris])
    floor = np.all(np.abs(v[:, 1::3] - (LO[1] + off[1])) < 1e-12, axis=1)
    return v, nrm, floor


def sample(x, v, w, r, m, floor_y):
    """(kinetic energy, coordination, packing) of one bed's state."""
    from scipy.spatial import cKDTree
    ke = float((0.5 * m * (v ** 2).sum(1)).sum() + (0.5 * 0.4 * m * r * r * (w ** 2).sum(1)).sum())
    pairs = cKDTree(x).query_pairs(2.0 * RMAX, output_type="ndarray")
    d = np.linalg.norm(x[pairs[:, 0]] - x[pairs[:, 1]], axis=1)
    z = 2.0 * float(np.count_nonzero(d < r[pairs[:, 0]] + r[pairs[:, 1]])) / len(r)
    top = np.percentile(x[:, 1] + r, 95)
    pack = float((4.0 / 3.0 * np.pi * r ** 3).sum() / (AREA * (top - floor_y)))
    return ke, z, pack


def sample_steps():
    return [s for s in range(EVERY, STEPS + 1, EVERY) if s > START]
