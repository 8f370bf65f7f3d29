"""Shared set-up for GPU-vs-oracle parity tests: seeded synthetic states, one
step on each side from the same state, and the comparisons."""
from collections import Counter

import numpy as np

NORMAL_NAMES = {0: "linear", 1: "hertz", 2: "hysteretic", 3: "jkr", 4: "sjkr"}
TANGENTIAL_NAMES = {0: "coulomb", 1: "linear", 2: "mindlin"}


def random_bed(seed, n, lo, hi, rmin, rmax, vscale=0.05, wscale=1.0, ascale=1.0, tscale=1e-6, fixed_frac=0.0,
               outside=0, jitter=0.02):
    """Particles on a jittered lattice filling [lo, hi] so that neighbours touch
    (overlaps up to a few % of a radius), with random v, omega, a, tau."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    # per-axis spacing that divides the box exactly, so a periodic face is
    # seamless; sites fill the box from the bottom (y) up, as a settled bed
    s0 = rmin + rmax  # about half of the neighbour pairs overlap
    dims = np.maximum(np.ceil((hi - lo) / s0).astype(int), 1)
    spacing = (hi - lo) / dims
    g = np.stack(np.meshgrid(*[np.arange(d) for d in dims], indexing="ij"), -1).reshape(-1, 3)
    g = g[np.lexsort((g[:, 2], g[:, 0], g[:, 1]))]
    g = g[:n]
    x = lo + (g + 0.5) * spacing + rng.uniform(-jitter, jitter, g.shape) * rmax
    k = len(x)
    r = rng.uniform(rmin, rmax, k)
    st = {
        "position": x,
        "radius": r,
        "mass": 2500.0 * 4.0 / 3.0 * np.pi * r ** 3,
        "velocity": rng.normal(0, vscale, (k, 3)),
        "angular_velocity": rng.normal(0, wscale, (k, 3)),
        "acceleration": rng.normal(0, ascale, (k, 3)),
        "torque": rng.normal(0, tscale, (k, 3)),
        "fixed": (rng.uniform(0, 1, k) < fixed_frac).astype(np.uint8),
    }
    if outside:
        # a few particles outside the box (reference grid does not insert them)
        idx = rng.choice(k, size=min(outside, k), replace=False)
        st["position"][idx] = hi + rng.uniform(0.0, 0.5, (len(idx), 3))
    return st


def oracle_sim(oracle_mod, st, dt, lo, hi, normal, tangential, periodic=(False, False, False), mode=0,
               material=(1e7, 0.3, 2500.0, 0.5, 0.5, 0.0), wall=None, tris=None, cell=1.0):
    s = oracle_mod.OracleSimulation(dt, lo, hi, prec=64)
    s.set_mode(mode)
    s.set_cell_size(cell)
    s.set_options(record_pairs=True, keep_contact_map=False)
    s.set_particle_material(*material)
    if wall is not None:
        s.set_wall_material(*wall)
    s._L.orc_set_models(s._h, normal, tangential)
    s.set_periodic_boundary(*periodic)
    for i in range(len(st["radius"])):
        p = st["position"][i]
        s.add_particle(p[0], p[1], p[2], st["radius"][i], st["mass"][i], bool(st["fixed"][i]))
    if tris is not None:
        s.add_triangles(tris[0], tris[1])
    s.set_state({"x": st["position"], "v": st["velocity"], "a": st["acceleration"], "w": st["angular_velocity"],
                 "tau": st["torque"]})
    return s


def gpu_sim(rp, st, dt, lo, hi, normal, tangential, periodic=(False, False, False), mode=0,
            material=(1e7, 0.3, 2500.0, 0.5, 0.5, 0.0), wall=None, tris=None, cell=1.0, precision=0, force_path=0):
    s = rp.Simulation.create(dt, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], len(st["radius"]))
    s._L.rp_set_force_path(s._h, force_path)
    s.set_interaction_mode(mode)
    s.set_precision(precision)
    s.set_reference_cell_size(cell)
    s.set_particle_material(*material)
    if wall is not None:
        s.set_wall_material(*wall)
    s.set_contact_models(NORMAL_NAMES[normal], TANGENTIAL_NAMES[tangential])
    s.set_periodic_boundary(*periodic)
    s.add_particles(st["position"], st["radius"], st["mass"], st["fixed"])
    if tris is not None:
        s.add_triangles(tris[0], tris[1])
    s.set_state({k: st[k] for k in ("velocity", "angular_velocity", "acceleration", "torque")})
    s.set_debug(True)
    return s


def pair_counter_oracle(o):
    pi, pj = o.pairs()
    return Counter(zip(pi.tolist(), pj.tolist()))


def pair_counter_gpu(g):
    pi, pj, vv = g.debug_pairs()
    c = Counter()
    for a, b, v in zip(pi.tolist(), pj.tolist(), vv.tolist()):
        c[(a, b)] += v
    return c


def rel_err(a, b, floor):
    """max_i |a_i - b_i| / max(|b_i|, floor) over particles (rows)."""
    d = np.linalg.norm(a - b, axis=1)
    s = np.maximum(np.linalg.norm(b, axis=1), floor)
    return float(np.max(d / s)) if len(d) else 0.0
