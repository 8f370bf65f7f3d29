#!/usr/bin/env python
"""Benchmark of the DEM step: particle-steps/s on one GB300.

Default workload (the configuration the metric is quoted on): 1,048,576
polydisperse spheres (radii lognormal, median 2 mm, sigma 0.25, clipped to
[1, 4] mm) packed to solid fraction ~0.55 inside a procedurally tessellated
conical hopper of 20,000 triangles (half-angle 30 deg, outlet radius 10 median
radii) above a floor at y = 0, periodic in x and z, Hertz + Mindlin, FP64,
dt = 2e-6 s. The packing is a seeded FCC start relaxed by grow-and-settle
stages run on the product engine before timing (not timed).

`value` is device time over the timed steps (inputs resident in HBM; the
state is larger than L2 so every step streams it from HBM). `e2e` is the
same metric through the public API with host buffers: state upload, K steps
and state read-back inside the timed region. `--impl reference` times the
reference algorithm on the host cores (the oracle's restatement of
`step_cpu`, literal 1 m grid and every-triangle wall loop, all threads) on a
bounded sample of the same workload.

Multi-GPU: the step does not shard (one bed per device); `--gpus N` under
torchrun runs one independent replica per rank (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300, plain vs learned-JKR/batched/FP32, at stated force error"
UNIT = "particle-steps/s"
# Algorithmic bytes per particle-step of the FP64 step: read own x, v, omega
# (72 B) + radius, mass (16 B), write x, v, omega (72 B).
B0_FP64 = 160.0
# Mindlin tangential spring (physical mode): 24 B read + written per pair.
B_HIST_PAIR = 48.0
B_TRIANGLE = 72.0


# ----------------------------------------------------------------- workloads
def cone_triangles(r_out, y_out, height, half_angle_deg, n_theta, n_y):
    """Frustum wall y in [y_out, y_out+height], radius r_out + (y-y_out) tan(a),
    n_theta x n_y quads split into 2 triangles, normals pointing inward."""
    t = math.tan(math.radians(half_angle_deg))
    th = np.linspace(0.0, 2.0 * np.pi, n_theta + 1)
    ys = np.linspace(y_out, y_out + height, n_y + 1)
    tris = []
    for j in range(n_y):
        y0, y1 = ys[j], ys[j + 1]
        r0, r1 = r_out + (y0 - y_out) * t, r_out + (y1 - y_out) * t
        for i in range(n_theta):
            a0, a1 = th[i], th[i + 1]
            p00 = (r0 * math.cos(a0), y0, r0 * math.sin(a0))
            p01 = (r0 * math.cos(a1), y0, r0 * math.sin(a1))
            p10 = (r1 * math.cos(a0), y1, r1 * math.sin(a0))
            p11 = (r1 * math.cos(a1), y1, r1 * math.sin(a1))
            tris.append((p00, p10, p01))
            tris.append((p01, p10, p11))
    v = np.asarray(tris, np.float64).reshape(-1, 9)
    a, b, c = v[:, 0:3], v[:, 3:6], v[:, 6:9]
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    centre = (a + b + c) / 3.0
    inward = np.stack([-centre[:, 0], np.zeros(len(v)), -centre[:, 2]], 1)
    flip = (n * inward).sum(1) < 0
    v[flip] = np.concatenate([a[flip], c[flip], b[flip]], 1)
    n[flip] = -n[flip]
    return v.astype(np.float32), n.astype(np.float32)


def floor_triangles(lo, hi, y=0.0):
    x0, z0, x1, z1 = lo[0], lo[2], hi[0], hi[2]
    v = np.array([[x0, y, z0, x0, y, z1, x1, y, z0], [x1, y, z0, x0, y, z1, x1, y, z1]], np.float32)
    n = np.array([[0, 1, 0], [0, 1, 0]], np.float32)
    return v, n


def hopper_workload(n=1_048_576, seed=2026, phi=0.55):
    """Hopper bed (see module docstring). Returns a dict with bounds, mesh and
    an FCC start state (radii at full size; overlaps removed by `relax`)."""
    rng = np.random.default_rng(seed)
    r = np.clip(rng.lognormal(np.log(2e-3), 0.25, n), 1e-3, 4e-3)
    rho = 2500.0
    v_bed = float((4.0 / 3.0 * np.pi * r ** 3).sum()) / phi
    t30 = math.tan(math.radians(30.0))
    r_out, y_out = 10 * 2e-3, 0.15

    def frustum(h):
        R = r_out + h * t30
        return math.pi / 3.0 * h * (R * R + R * r_out + r_out * r_out)

    lo_h, hi_h = 0.0, 5.0
    for _ in range(80):
        mid = 0.5 * (lo_h + hi_h)
        lo_h, hi_h = (mid, hi_h) if frustum(mid) < v_bed else (lo_h, mid)
    h_fill = hi_h
    h_cone = h_fill * 1.15 + 0.02
    R_top = r_out + h_cone * t30
    half = round(R_top + 0.05, 2)
    lo = (-half, 0.0, -half)
    hi = (half, round(y_out + h_cone + 0.1, 2), half)
    # FCC sites at the bed's number density inside the cone (margin from wall)
    a = (4.0 * v_bed / n) ** (1.0 / 3.0)
    margin = 2e-3
    for _ in range(20):
        k = np.arange(-math.ceil(R_top / a) - 1, math.ceil(R_top / a) + 2)
        ky = np.arange(0, math.ceil(h_cone / a) + 1)
        base = np.stack(np.meshgrid(k, ky, k, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
        offs = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
        sites = (base[:, None, :] + offs[None]).reshape(-1, 3) * a
        sites[:, 1] += y_out + margin
        rho_s = np.hypot(sites[:, 0], sites[:, 2])
        inside = (rho_s < r_out + (sites[:, 1] - y_out) * t30 - margin) & (sites[:, 1] < y_out + h_cone - margin)
        sites = sites[inside]
        if len(sites) >= n:
            break
        a *= 0.98
    sites = sites[np.argsort(sites[:, 1], kind="stable")][:n]
    x = sites + rng.uniform(-0.02, 0.02, sites.shape) * a
    cv, cn = cone_triangles(r_out, y_out, h_cone, 30.0, 100, 100)
    fv, fn = floor_triangles(lo, hi)
    return {
        "name": "hopper-1M", "settle": 2000,
        # Verlet skin of the neighbour lists (a margin of this engine, not of the
        # reference's algorithm; results do not depend on it): 0.4 mm measured
        # fastest on this bed over 0.3-0.8 mm (the default, 0.2 of the largest
        # radius, would be 0.8 mm)
        "skin": 4e-4,
        "lo": lo, "hi": hi, "periodic": (True, False, True),
        "dt": 2e-6, "normal": "hertz", "tangential": "mindlin",
        "material": (1e7, 0.3, rho, 0.5, 0.5, 0.0),
        "tri_v": np.concatenate([fv, cv]), "tri_n": np.concatenate([fn, cn]),
        "position": x, "radius": r, "mass": rho * 4.0 / 3.0 * np.pi * r ** 3,
        "describe": (f"{n:,} spheres, radii lognormal (median 2 mm, sigma 0.25, clipped [1,4] mm), solid fraction "
                     f"{phi} in a 30-deg conical hopper (outlet radius 20 mm, {len(cv):,} triangles) over a floor, "
                     "periodic x/z, Hertz+Mindlin, dt=2e-6 s"),
    }


def box_workload(seed=7):
    """1,000 spheres on a jittered 10x10x10 lattice in [-1,1]^3 (spacing 0.2,
    jitter <= 0.05), radii U[0.01, 0.02], reflecting walls as a 12-triangle box
    mesh, Hertz+Coulomb, E=1e7, nu=0.3, rho=2500, e=0.5, mu=0.5, dt=1e-5."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(10)] * 3, indexing="ij"), -1).reshape(-1, 3)
    x = -0.9 + 0.2 * g + rng.uniform(-0.05, 0.05, g.shape)
    r = rng.uniform(0.01, 0.02, len(x))
    from tests.stl_util import box_tris
    tris = box_tris((-1, -1, -1), (1, 1, 1))
    v = np.array([np.concatenate(t) for t in tris], np.float32)
    n = np.array([np.cross(t[1] - t[0], t[2] - t[0]) / np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0]))
                  for t in tris], np.float32)
    return {
        "name": "box-1k", "lo": (-1.0, -1.0, -1.0), "hi": (1.0, 1.0, 1.0), "periodic": (False, False, False),
        "dt": 1e-5, "normal": "hertz", "tangential": "coulomb", "material": (1e7, 0.3, 2500.0, 0.5, 0.5, 0.0),
        "tri_v": v, "tri_n": n, "position": x, "radius": r, "mass": 2500.0 * 4.0 / 3.0 * np.pi * r ** 3,
        "describe": "1,000 spheres, jittered 10^3 lattice in [-1,1]^3, radii U[0.01,0.02], 12-triangle box walls, "
                    "Hertz+Coulomb, dt=1e-5 s",
    }


def adhesive_workload(n=4_194_304, seed=2027, phi=0.35):
    """Adhesive gas: n spheres, radii U[5, 20] um, JKR + Coulomb, E = 5e8 Pa,
    nu = 0.25, surface energy 0.05 J/m^2, rho = 2000 kg/m^3, in a periodic cube
    at solid fraction 0.35 with Gaussian velocities (sigma 0.05 m/s per axis),
    dt = 1e-8 s. Start: a shuffled cubic lattice at 0.6x radii grown to full
    size by `relax` (no overlaps at the start of the timed run)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(5e-6, 20e-6, n)
    rho = 2000.0
    L = (float((4.0 / 3.0 * np.pi * r ** 3).sum()) / phi) ** (1.0 / 3.0)
    m = math.ceil(n ** (1.0 / 3.0))
    s = L / m
    g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
    g = g[rng.permutation(len(g))[:n]]
    g = g[np.lexsort((g[:, 2], g[:, 1], g[:, 0]))]
    x = (g + 0.5) * s + rng.uniform(-0.05, 0.05, g.shape) * s
    return {
        "name": "adhesive-4M" if n == 4_194_304 else f"adhesive-{n}", "settle": 1600,
        "lo": (0.0, 0.0, 0.0), "hi": (L, L, L), "periodic": (True, True, True),
        "dt": 1e-8, "normal": "jkr", "tangential": "coulomb",
        "material": (5e8, 0.25, rho, 0.5, 0.5, 0.05),
        "tri_v": np.zeros((0, 9), np.float32), "tri_n": np.zeros((0, 3), np.float32),
        "position": x, "radius": r, "mass": rho * 4.0 / 3.0 * np.pi * r ** 3,
        "velocity": rng.normal(0.0, 0.05, (n, 3)),
        "describe": (f"{n:,} spheres, radii U[5,20] um, JKR+Coulomb, E=5e8 Pa, nu=0.25, gamma=0.05 J/m^2, "
                     f"rho=2000, periodic cube L={L * 1e3:.3f} mm at solid fraction {phi}, Gaussian velocities "
                     "(sigma 0.05 m/s), dt=1e-8 s"),
    }


def batched_workload(n_boxes=512, seed=2028, phi=0.45, n_lo=2000, n_hi=60000):
    """n_boxes independent walled boxes, each with a particle count drawn
    log-uniform in [n_lo, n_hi], radii U[0.5, 1.5] mm, sJKR + Coulomb,
    surface energy U[0, 0.1] J/m^2 per box (E = 1e7 Pa, nu = 0.3, rho = 2500,
    mu = 0.5, e = 0.5), box side giving solid fraction phi, dt = 1e-6 s; the
    boxes sit on an 8 x 8 x 8 grid of slots with gaps wider than any cutoff.
    Each box is one group (its own bed, material and 12 wall triangles)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), n_boxes)).astype(np.int64)
    gammas = rng.uniform(0.0, 0.1, n_boxes)
    radii = [rng.uniform(0.5e-3, 1.5e-3, c) for c in counts]
    sides = np.array([(float((4.0 / 3.0 * np.pi * r ** 3).sum()) / phi) ** (1.0 / 3.0) for r in radii])
    slot = float(sides.max()) + 0.006
    per = math.ceil(n_boxes ** (1.0 / 3.0))
    from tests.stl_util import box_tris
    xs, rs, gs, tv, tn, tg = [], [], [], [], [], []
    for b in range(n_boxes):
        i, j, k = b % per, (b // per) % per, b // (per * per)
        lo = np.array([i, j, k], float) * slot + 0.003
        side = sides[b]
        m = math.ceil(counts[b] ** (1.0 / 3.0))
        sp = side / m
        g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
        g = g[rng.permutation(len(g))[:counts[b]]]
        g = g[np.lexsort((g[:, 2], g[:, 0], g[:, 1]))]
        xs.append(lo + (g + 0.5) * sp)
        rs.append(radii[b])
        gs.append(np.full(counts[b], b, np.uint32))
        for t in box_tris(lo, lo + side):
            nv = np.cross(t[1] - t[0], t[2] - t[0])
            tv.append(np.concatenate(t))
            tn.append(nv / np.linalg.norm(nv))
            tg.append(b)
    r = np.concatenate(rs)
    top = per * slot + 0.006
    return {
        "name": f"batched-{n_boxes}", "settle": 1200, "lo": (0.0, 0.0, 0.0), "hi": (top, top, top), "periodic": (False, False, False),
        "dt": 1e-6, "normal": "sjkr", "tangential": "coulomb", "material": (1e7, 0.3, 2500.0, 0.5, 0.5, gammas[0]),
        "tri_v": np.asarray(tv, np.float32), "tri_n": np.asarray(tn, np.float32), "tri_group": np.asarray(tg),
        "position": np.concatenate(xs), "radius": r, "mass": 2500.0 * 4.0 / 3.0 * np.pi * r ** 3,
        "groups": np.concatenate(gs), "counts": counts,
        "group_material": [(1e7, 0.3, 2500.0, 0.5, 0.5, float(gm)) for gm in gammas],
        "describe": (f"{n_boxes} independent walled boxes, {int(counts.sum()):,} spheres in all (per box log-uniform "
                     f"in [{n_lo:,}, {n_hi:,}]), radii U[0.5,1.5] mm, sJKR+Coulomb, surface energy U[0,0.1] J/m^2 "
                     f"per box, solid fraction {phi}, dt=1e-6 s, all boxes stepped by one device loop"),
    }


def drum_triangles(R, L, n_theta=256, n_z=117, n_rings=5):
    """Closed cylinder about the z axis (radius R, z in [0, L]): n_theta x n_z
    wall quads, and per end cap a 256-triangle fan plus n_rings rings of
    n_theta quads; normals point inward. 256*117*2 + 2*256*11 = 65,536."""
    th = np.linspace(0.0, 2.0 * np.pi, n_theta + 1)
    zs = np.linspace(0.0, L, n_z + 1)
    c, s = np.cos(th), np.sin(th)
    tris = []
    for j in range(n_z):
        for i in range(n_theta):
            p00 = (R * c[i], R * s[i], zs[j]); p01 = (R * c[i + 1], R * s[i + 1], zs[j])
            p10 = (R * c[i], R * s[i], zs[j + 1]); p11 = (R * c[i + 1], R * s[i + 1], zs[j + 1])
            tris += [(p00, p01, p10), (p01, p11, p10)]
    rr = np.linspace(0.0, R, n_rings + 2)
    for z in (0.0, L):
        for i in range(n_theta):
            tris.append(((0.0, 0.0, z), (rr[1] * c[i], rr[1] * s[i], z), (rr[1] * c[i + 1], rr[1] * s[i + 1], z)))
        for k in range(1, n_rings + 1):
            for i in range(n_theta):
                a0 = (rr[k] * c[i], rr[k] * s[i], z); a1 = (rr[k] * c[i + 1], rr[k] * s[i + 1], z)
                b0 = (rr[k + 1] * c[i], rr[k + 1] * s[i], z); b1 = (rr[k + 1] * c[i + 1], rr[k + 1] * s[i + 1], z)
                tris += [(a0, b0, a1), (a1, b0, b1)]
    v = np.asarray(tris, np.float64).reshape(-1, 9)
    a, b, cc = v[:, 0:3], v[:, 3:6], v[:, 6:9]
    n = np.cross(b - a, cc - a)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    centre = (a + b + cc) / 3.0
    inward = np.stack([-centre[:, 0], -centre[:, 1], L / 2 - centre[:, 2]], 1)
    flip = (n * inward).sum(1) < 0
    v[flip] = np.concatenate([a[flip], cc[flip], b[flip]], 1)
    n[flip] = -n[flip]
    return v.astype(np.float32), n.astype(np.float32)


def drum_workload(n=16_777_216, seed=2029, R=0.5, rpm=30.0, fill=0.4):
    """Rotating drum: n spheres, radii U[1, 2] mm, Hertz + Coulomb, E = 1e7 Pa,
    nu = 0.3, rho = 2500, restitution 0.3, friction 0.4, in a closed drum of
    radius R about the z axis turning at `rpm` (the 65,536-triangle wall moves
    with omega x p), filled to `fill` of its volume, dt = 5e-6 s. The drum
    length follows from the fill: n spheres of this size fill 40 % of a
    0.5 m x 1.7 m drum (a 0.3 m drum holds about 3.5 M of them). Start: a
    shuffled cubic lattice in the lower segment at 0.6x radii grown by `relax`."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(1e-3, 2e-3, n)
    sp = (float((4.0 / 3.0 * np.pi * r ** 3).mean()) / 0.5) ** (1.0 / 3.0)  # lattice at solid fraction 0.5
    area = fill * np.pi * R * R
    lo_y, hi_y = -R, R
    for _ in range(80):  # fill height of the circular segment with that area
        y = 0.5 * (lo_y + hi_y)
        seg = R * R * math.acos(-y / R) + y * math.sqrt(max(R * R - y * y, 0.0))
        lo_y, hi_y = (y, hi_y) if seg < area else (lo_y, y)
    yf = 0.5 * (lo_y + hi_y)
    rin = R - 2.5e-3
    kx = np.arange(-math.ceil(R / sp), math.ceil(R / sp) + 1)
    gx, gy = np.meshgrid(kx * sp, kx * sp, indexing="ij")
    ok = (gx ** 2 + gy ** 2 < rin ** 2) & (gy < yf)
    xy = np.stack([gx[ok], gy[ok]], 1)
    layers = math.ceil(n / len(xy))
    L = layers * sp + 6e-3
    z = 3e-3 + (np.arange(layers) + 0.5) * sp
    sites = np.concatenate([np.column_stack([xy, np.full(len(xy), zz)]) for zz in z])
    sites = sites[rng.permutation(len(sites))[:n]]
    sites = sites[np.lexsort((sites[:, 0], sites[:, 1], sites[:, 2]))]
    x = sites + rng.uniform(-0.02, 0.02, sites.shape) * sp
    v, nn = drum_triangles(R, L)
    w = 2.0 * np.pi * rpm / 60.0
    m = 0.02
    return {
        "name": "drum-16M" if n == 16_777_216 else f"drum-{n}", "settle": 600,
        "lo": (-R - m, -R - m, -m), "hi": (R + m, R + m, L + m), "periodic": (False, False, False),
        "dt": 5e-6, "normal": "hertz", "tangential": "coulomb", "material": (1e7, 0.3, 2500.0, 0.4, 0.3, 0.0),
        "tri_v": v, "tri_n": nn, "tri_motion": ((0.0, 0.0, 0.0), (0.0, 0.0, w), (0.0, 0.0, 0.0)),
        "position": x, "radius": r, "mass": 2500.0 * 4.0 / 3.0 * np.pi * r ** 3,
        "describe": (f"{n:,} spheres, radii U[1,2] mm, Hertz+Coulomb, E=1e7 Pa, e=0.3, mu=0.4, rotating drum "
                     f"R={R} m x L={L:.2f} m ({len(v):,} triangles, {rpm:g} rpm about z), fill {fill}, dt=5e-6 s"),
    }


def make_workload(args):
    if args.workload == "drum":
        return drum_workload(n=args.particles or 16_777_216)
    if args.workload == "batched":
        return batched_workload(n_boxes=args.boxes)
    if args.workload == "hopper":
        return hopper_workload(n=args.particles or 1_048_576)
    if args.workload == "adhesive":
        return adhesive_workload(n=args.particles or 4_194_304)
    return box_workload()


def make_sim(rp, wl, mode="parity", precision="fp64"):
    lo, hi = wl["lo"], wl["hi"]
    s = rp.Simulation.create(wl["dt"], lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], len(wl["radius"]))
    s.set_interaction_mode(mode)
    s.set_precision(precision)
    s.set_particle_material(*wl["material"])
    s.set_contact_models(wl["normal"], wl["tangential"])
    s.set_periodic_boundary(*wl["periodic"])
    if "tri_group" in wl:
        for g in range(len(wl["group_material"])):
            sel = wl["tri_group"] == g
            s.add_triangles(wl["tri_v"][sel], wl["tri_n"][sel], group=g)
    elif len(wl["tri_v"]):
        s.add_triangles(wl["tri_v"], wl["tri_n"], motion=wl.get("tri_motion"))
    s.add_particles(wl["position"], wl["radius"], wl["mass"])
    if "groups" in wl:
        s.set_particle_groups(wl["groups"])
        for g, m in enumerate(wl["group_material"]):
            s.set_group_material(g, *m)
    if "velocity" in wl:
        s.set_state({"velocity": wl["velocity"]})
    if wl.get("skin"):
        s.set_skin(wl["skin"])
    return s


def skin_of(wl, args):
    """The Verlet skin a timed simulation of `wl` runs with."""
    if getattr(args, "skin", None):
        return float(args.skin)
    if wl.get("skin"):
        return float(wl["skin"])
    return 0.2 * float(np.max(wl["radius"]))


def one_box_workload(wl, b):
    """Box b of a batched workload as its own single-group workload."""
    sel = wl["groups"] == b
    tsel = wl["tri_group"] == b
    return {
        "name": f"box-{b}", "lo": wl["lo"], "hi": wl["hi"], "periodic": wl["periodic"], "dt": wl["dt"],
        "normal": wl["normal"], "tangential": wl["tangential"], "material": wl["group_material"][b],
        "tri_v": wl["tri_v"][tsel], "tri_n": wl["tri_n"][tsel], "position": wl["position"][sel],
        "radius": wl["radius"][sel], "mass": wl["mass"][sel],
    }


def one_at_a_time(rp, wl, steps, n_sample=16, log=None):
    """Particle-steps/s when the boxes are stepped as separate simulations (one
    device loop per box, same engine), on a sample of boxes spread over the
    size range, extrapolated by total particle-steps over total device time."""
    order = np.argsort(wl["counts"], kind="stable")
    pick = order[np.linspace(0, len(order) - 1, min(n_sample, len(order))).astype(int)]
    units, ms = 0, 0.0
    for b in pick:
        s = make_sim(rp, one_box_workload(wl, int(b)))
        s.steps(int(wl.get("settle", 0)) + 3)  # settled as the batched run
        a = s.stats()
        s.steps(steps)
        c = s.stats()
        units += int(c["particles"]) * steps
        ms += c["device_ms"] - a["device_ms"]
        del s
    return {"value": units / (ms / 1e3), "boxes_timed": int(len(pick)), "steps_each": steps,
            "sample": "boxes at evenly spaced size quantiles, each its own Simulation (device loop)"}


def relax(rp, wl, stages=9, steps_per_stage=100, settle=300, log=None):
    """Grow radii from 0.6x to 1x in stages while a damped, frictionless,
    gravity-free run removes the overlaps; updates wl["position"] in place.
    The time step scales with the smallest radius (1e-5 s at 1 mm)."""
    x = wl["position"].copy()
    r, m = wl["radius"], wl["mass"]
    lo, hi = wl["lo"], wl["hi"]
    dt = 1e-5 * float(np.min(r)) / 1e-3
    s = rp.Simulation.create(dt, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], len(r))
    s.set_interaction_mode("parity")
    s.set_particle_material(1e7, 0.3, 2500.0, 0.0, 0.05, 0.0)
    s.set_contact_models("hertz", "coulomb")
    s.set_periodic_boundary(*wl["periodic"])
    s.set_gravity(0.0, 0.0, 0.0)
    if len(wl["tri_v"]):
        s.add_triangles(wl["tri_v"], wl["tri_n"])
    s.add_particles(x, r * 0.6, m * 0.216)
    t0 = time.time()
    for k, f in enumerate(np.linspace(0.6, 1.0, stages)):
        st = {"radius": r * f, "mass": m * f ** 3, "velocity": np.zeros_like(x), "angular_velocity": np.zeros_like(x),
              "acceleration": np.zeros_like(x), "torque": np.zeros_like(x)}
        s.set_state(st)
        s.steps(steps_per_stage if k < stages - 1 else settle)
    out = s.get_state()
    if len(out["radius"]) != len(r):
        raise RuntimeError(f"relaxation lost particles ({len(out['radius'])} of {len(r)})")
    wl["position"] = out["position"]
    if log:
        log(f"relaxed {len(r):,} particles in {time.time() - t0:.1f} s")
    return wl


# ------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [q.strip() for q in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers
def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def allreduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(workload_name, n):
    """DRAM bytes of one force pass (all its kernels) from the committed ncu
    summary (profiles/force_pass_<workload>.json, captured on a smaller bed of
    the same workload), scaled to n particles (traffic grows with the units),
    and the FP64-pipe activity of its kernels from the same captures."""
    p = os.path.join(ROOT, "profiles", f"force_pass_{workload_name}.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_pass"]) * n / float(d["particles"]), d.get("fp64_pipe_active_pct")
    except (OSError, KeyError, ValueError):
        return None, None


_FP64_PEAK = {}


def fp64_roofline(rp, wl, n, ms_per_step, suffix=""):
    """The step against the FP64 pipe: the device's FP64 rate measured by
    librp (rp_measure_fp64_peak, once per run), the FP64-pipe thread
    instructions per particle-step counted by ncu on a smaller bed of the same
    workload and form (profiles/fp64_ops_<workload><suffix>.json), and the
    fraction of that rate the timed step reaches."""
    import ctypes
    from rusty_particles_gb300 import _lib
    if not _FP64_PEAK:
        fma, add = ctypes.c_double(), ctypes.c_double()
        if _lib.load().rp_measure_fp64_peak(ctypes.byref(fma), ctypes.byref(add)) != 0:
            return None
        _FP64_PEAK.update(fma=fma.value, add=add.value)
    fma = ctypes.c_double(_FP64_PEAK["fma"])
    out = {"peak_fma_per_s": _FP64_PEAK["fma"], "peak_add_per_s": _FP64_PEAK["add"],
           "unit": "FP64 thread instructions/s",
           "peak_source": "measured in this run (librp rp_measure_fp64_peak, CUDA events)"}
    p = os.path.join(ROOT, "profiles", f"fp64_ops_{wl['name']}{suffix}.json")
    try:
        with open(p) as f:
            d = json.load(f)
        per = float(d["fp64_pipe_inst_per_particle_step"])
    except (OSError, KeyError, ValueError):
        return out
    achieved = per * n / (ms_per_step / 1e3)
    out.update({"fp64_pipe_inst_per_particle_step": per,
                "dadd_dmul_dfma_per_particle_step": d.get("dadd_dmul_dfma_per_particle_step"),
                "achieved": achieved, "frac": achieved / fma.value,
                "counts_source": d.get("source")})
    return out


# ------------------------------------------------------ CPU side (the oracle)
STATE_VEC = ("position", "velocity", "angular_velocity", "acceleration", "torque", "position_residual",
             "velocity_residual", "angular_velocity_residual")
ORACLE_KEYS = {"position": "x", "velocity": "v", "acceleration": "a", "angular_velocity": "w", "torque": "tau",
               "position_residual": "xres", "velocity_residual": "vres", "angular_velocity_residual": "wres"}


def max_cutoff(wl):
    """The largest pair cutoff of the workload: 2 r_max, times 1.5 for the
    adhesive laws (the reference's margin, src/simulation.rs:343-357)."""
    adh = 1.5 if wl["normal"] in ("jkr", "sjkr") else 1.0
    return 2.0 * float(np.max(wl["radius"])) * adh


def cpu_sample(wl, n_sample, seed=3):
    """A compact sub-block of the bed: the n_sample particles nearest the bed's
    centre of mass, with the workload's full mesh."""
    x = wl["position"]
    c = x.mean(0)
    idx = np.argsort(np.linalg.norm(x - c, axis=1), kind="stable")[:n_sample]
    idx.sort()
    return idx


def oracle_for(wl, state=None, prec=64, cell=1.0, cull=False, idx=None, mode=0, material=None, tri_sel=None):
    """The oracle on the workload (or the particles idx of it), from `state`
    (arrays as get_state returns them) or from the workload's start."""
    from oracle import oracle as om
    om.build()
    lo, hi = wl["lo"], wl["hi"]
    o = om.OracleSimulation(wl["dt"], lo, hi, prec=prec)
    o.set_mode(mode)
    o.set_cell_size(cell)
    o.set_options(record_pairs=False, keep_contact_map=True)
    o.set_particle_material(*(material or wl["material"]))
    o.set_contact_models(wl["normal"], wl["tangential"])
    o.set_periodic_boundary(*wl["periodic"])
    src = state if state is not None else {"position": wl["position"], "radius": wl["radius"], "mass": wl["mass"]}
    sel = slice(None) if idx is None else idx
    o.add_particles(src["position"][sel], src["radius"][sel], src["mass"][sel])
    tv, tn = wl["tri_v"], wl["tri_n"]
    if tri_sel is not None:
        tv, tn = tv[tri_sel], tn[tri_sel]
    if len(tv):
        o.add_triangles(tv.astype(np.float64), tn.astype(np.float64), motion=wl.get("tri_motion"))
    o.set_wall_cull(cull)
    if state is not None:
        o.set_state({ORACLE_KEYS[k]: state[k][sel] for k in STATE_VEC if k in state})
    elif "velocity" in wl:
        o.set_state({"v": wl["velocity"][sel]})
    return o


def time_oracle(o, n, budget_s, max_steps=200, min_steps=1):
    """Steps `o` for about budget_s (after one untimed step); particle-steps/s."""
    t0 = time.perf_counter()
    o.steps(1)
    t1 = time.perf_counter() - t0
    steps = max(min_steps, min(max_steps, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.steps(steps)
    dt = time.perf_counter() - t0
    return n * steps / dt, steps, dt


def compare_forces(Fg, Tg, Fo, To, FS, TS, net_floor=1e-3):
    """Per-particle force and torque errors of one step against the FP64
    oracle: max |dF_i| / sum_j |f_ij| (the rounding scale of a reordered sum)
    and max |dF_i| / |F_i| over the particles whose net force is not a
    near-cancellation (|F_i| >= net_floor sum_j |f_ij|)."""
    out = {"particles": int(len(Fo))}
    fin = np.isfinite(Fo).all(1) & np.isfinite(To).all(1)
    out["nonfinite_mismatch"] = int(np.count_nonzero(fin != (np.isfinite(Fg).all(1) & np.isfinite(Tg).all(1))))
    for tag, G, O, S in (("force", Fg, Fo, FS), ("torque", Tg, To, TS)):
        d = np.linalg.norm(G - O, axis=1)[fin]
        s = S[fin]
        net = np.linalg.norm(O, axis=1)[fin]
        pos = s > 0
        out[f"{tag}_rel_sum"] = float(np.max(d[pos] / s[pos], initial=0.0))
        out[f"{tag}_abs_where_zero_scale"] = float(np.max(d[~pos], initial=0.0))
        sel = pos & (net >= net_floor * s)
        out[f"{tag}_rel_net"] = float(np.max(d[sel] / net[sel], initial=0.0))
        out[f"{tag}_net_counted"] = int(np.count_nonzero(sel))
    out["scales"] = (f"rel_sum: |dF_i| / sum_j |f_ij| (per-contact term magnitudes); rel_net: |dF_i| / |F_i| "
                     f"where |F_i| >= {net_floor:g} sum_j |f_ij|")
    return out


# ------------------------------------------------------------------- GPU side
def state_of(sim):
    return sim.get_state()


def wl_at(wl, state):
    """The workload with its particles at `state` (same radii, masses)."""
    w = dict(wl)
    w["position"] = state["position"]
    w["radius"] = state["radius"]
    w["mass"] = state["mass"]
    w.pop("velocity", None)
    return w


def set_dynamic_state(sim, state):
    sim.set_state({k: state[k] for k in STATE_VEC if k != "position" and k in state})


def setup_jkr(sim, jkr):
    if not jkr:
        return
    if jkr["solver"] == "learned":
        sim.set_jkr_network(*jkr["network"])
    sim.set_jkr_solver(jkr["solver"])


def gpu_one_step_forces(rp, wl, state, mode, precision, jkr, cell):
    """One GPU step from `state` with debug recording and the reference grid
    cell `cell`; (F, T) per particle in id order, before division by mass."""
    g = make_sim(rp, wl_at(wl, state), mode, precision)
    g.set_reference_cell_size(cell)
    setup_jkr(g, jkr)
    set_dynamic_state(g, state)
    g.set_debug(True)
    g.step()
    F, T = g.debug_forces()
    del g
    return F, T


def force_error(rp, wl, state, mode, precision, jkr, cache, log, threads, keep_oracle=False):
    """The form's one-step force error against the FP64 oracle on the full
    benchmark state: both sides step once from the same state with the
    reference grid's cell at the largest cutoff (the oracle's wall loop culled
    exactly). Batched workloads compare a sample of boxes, each against its own
    oracle (one reference Simulation per box)."""
    from oracle import oracle as om
    om.build()
    om.set_threads(threads)
    hc = max_cutoff(wl)
    t0 = time.perf_counter()
    Fg, Tg = gpu_one_step_forces(rp, wl, state, mode, precision, jkr, hc)
    t_gpu = time.perf_counter() - t0
    m = 0 if mode == "parity" else 1
    if "groups" in wl:
        order = np.argsort(wl["counts"], kind="stable")
        pick = order[np.linspace(0, len(order) - 1, min(8, len(order))).astype(int)]
        keys = []
        Fo_l, To_l, FS_l, TS_l, Fg_l, Tg_l = [], [], [], [], [], []
        t0 = time.perf_counter()
        for b in pick:
            idx = np.flatnonzero(wl["groups"] == b)
            key = ("box", wl["name"], int(b), m)
            if key not in cache:
                o = oracle_for(wl, state, cell=hc, cull=True, idx=idx, mode=m, material=wl["group_material"][b],
                               tri_sel=wl["tri_group"] == b)
                o.step()
                cache[key] = (*o.last_forces(), *o.last_force_scale())
                del o
            Fo, To, FS, TS = cache[key]
            Fo_l.append(Fo); To_l.append(To); FS_l.append(FS); TS_l.append(TS)
            Fg_l.append(Fg[idx]); Tg_l.append(Tg[idx])
            keys.append(int(b))
        t_or = time.perf_counter() - t0
        res = compare_forces(np.concatenate(Fg_l), np.concatenate(Tg_l), np.concatenate(Fo_l), np.concatenate(To_l),
                             np.concatenate(FS_l), np.concatenate(TS_l))
        res["boxes"] = keys
    else:
        key = (wl["name"], m)
        t0 = time.perf_counter()
        if key not in cache:
            o = oracle_for(wl, state, cell=hc, cull=True, mode=m)
            o.step()
            cache[key] = (*o.last_forces(), *o.last_force_scale())
            if keep_oracle:
                cache[key + ("oracle",)] = o  # kept for the CPU baseline timing
            del o
        t_or = time.perf_counter() - t0
        Fo, To, FS, TS = cache[key]
        res = compare_forces(Fg, Tg, Fo, To, FS, TS)
    res["method"] = (f"one step from the timed run's final state on both sides, reference-grid cell {hc * 1e3:.4g} mm "
                     "(the largest cutoff) on both" + (", spring history from zero on both" if mode == "physical"
                                                       else ""))
    res["seconds"] = {"gpu": round(t_gpu, 2), "oracle": round(t_or, 2)}
    log(f"force error {wl['name']} {mode}/{precision}{'/' + jkr['solver'] if jkr else ''}: "
        f"F {res['force_rel_sum']:.2e} (sum scale) {res['force_rel_net']:.2e} (net)")
    return res


def timed(sim, steps, dist, device):
    """K steps of the device step loop between barriers and synchronisations,
    with the clock sampler running; device ms from CUDA events on the
    engine's stream."""
    import torch
    torch.cuda.synchronize()
    s0 = sim.stats()
    clocks = ClockSampler(device)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    sim.steps(steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier(dist)
    ck = clocks.stop()
    s1 = sim.stats()
    return s0, s1, wall, ck


def roofline_of(sim, wl, n_now, prof_steps):
    """The force pass's roofline: the same steps issued from the host with
    CUDA events around every force launch on the engine's stream."""
    sim._L.rp_set_profiling(sim._h, 1)
    p0 = sim.stats()
    sim.steps(prof_steps)
    p1 = sim.stats()
    sim._L.rp_set_profiling(sim._h, 0)
    force_ms = (p1["force_ms"] - p0["force_ms"]) / max(1, p1["force_launches"] - p0["force_launches"])
    step_ms = (p1["device_ms"] - p0["device_ms"]) / max(1, p1["steps"] - p0["steps"])
    tri = len(wl["tri_v"])
    alg_bytes = n_now * B0_FP64 + tri * B_TRIANGLE
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (force_ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None,
            "kernel": ("force pass (k_contact_filter with the wall pretests, k_contact_force with the wall "
                       "contacts, k_accumulate)"),
            "avg_launch_ms": force_ms, "force_share_of_step": force_ms / step_ms if step_ms > 0 else None,
            "algorithmic_bytes_per_launch": alg_bytes, "peak_source": peak_kind}


def e2e_of(sim, n, steps, dist):
    """End to end through the public API with host buffers: set_state of the
    full state, K steps, get_state into arrays allocated before timing."""
    import torch
    st = sim.get_state()
    out_buf = {k: np.empty_like(v) for k, v in st.items()}
    for v in out_buf.values():
        v.fill(0)
    e0 = sim.stats()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.set_state(st)
    sim.steps(steps)
    sim.get_state(out=out_buf)
    wall = time.perf_counter() - t0
    dev_ms = sim.stats()["device_ms"] - e0["device_ms"]
    h2d = sum(int(v.nbytes) for v in st.values())
    d2h = sum(int(v.nbytes) for v in out_buf.values())
    val = allreduce_sum(dist, n * steps) / allreduce_max(dist, wall)
    return {"value": val, "unit": UNIT, "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "note": ("set_state (H2D of the full state) + steps(K) + get_state(out=...) (D2H into host arrays "
                     "allocated before timing), K = steps, run after the timed steps"),
            "device_ms_of_steps": dev_ms, "wall_ms": wall * 1e3,
            "transfer": ("kernels on the caller's pageable arrays" if sim.stats().get("state_io_direct")
                         else "one device copy per array, gather/scatter kernels between id order and the slots")}


def run_form(rp, wl, args, dist, device, log, *, mode="parity", precision="fp64", jkr=None, state=None, settle=0,
             steps=None, warmup=None, prof_steps=None, autotune=False, host_loop=False, keep=False):
    """One form of a workload: build the simulation (from `state` when given),
    untimed settle and warm-up steps, the timed steps, the force-pass roofline
    and the end-to-end run. Returns (sim or None, result, final state)."""
    steps = steps or args.steps
    warmup = max(3, warmup if warmup is not None else args.warmup)
    sim = make_sim(rp, wl if state is None else wl_at(wl, state), mode, precision)
    if getattr(args, "skin", None):
        sim.set_skin(args.skin)
    sim._L.rp_enable_gpu(sim._h, device)
    if host_loop:
        sim._L.rp_set_device_loop(sim._h, 0)
    setup_jkr(sim, jkr)
    if state is not None:
        set_dynamic_state(sim, state)
    if settle:
        t_settle = time.time()
        sim.steps(settle)
        log(f"{wl['name']} {mode}/{precision}: settled {settle} steps in {time.time() - t_settle:.1f} s")
    sim.steps(warmup)
    tune = sim.autotune() if autotune else None
    c0 = sim.jkr_counters() if jkr else None
    s0, s1, wall, ck = timed(sim, steps, dist, device)
    dev_ms = s1["device_ms"] - s0["device_ms"]
    n_now = s1["particles"]
    t_max = allreduce_max(dist, dev_ms)
    value = allreduce_sum(dist, n_now * steps) / (t_max / 1e3)
    res = {"value": value, "unit": UNIT, "ms_per_step": t_max / steps, "steps": steps, "warmup": warmup,
           "particles": int(n_now), "mode": mode, "precision": precision, "wall_s_timed": wall,
           "gpu_launches": int(s1["kernel_launches"] - s0["kernel_launches"]), "clocks": ck,
           "stats": {k: s1[k] for k in ("neighbor_rebuilds", "max_neighbors", "neighbor_capacity", "removed")},
           "verlet_skin_m": skin_of(wl, args)}
    if jkr:
        c1 = sim.jkr_counters()
        d = {k: (c1[k] - c0[k]) / steps for k in c1}
        ev = d["accepted"] + d["zero"] + d["fallback"]
        res["jkr"] = {"solver": jkr["solver"], "per_step": d}
        if ev > 0:
            res["jkr"]["fraction"] = {"converging": d["accepted"] / ev, "certified_zero": d["zero"] / ev,
                                      "reference_newton": d["fallback"] / ev}
    if tune:
        res["autotune"] = tune
    try:  # the timed state: kinetic energy, coordination number, solid fraction of the box
        res["bed"] = sim.bed_statistics()
    except Exception:  # noqa: BLE001 - a statistic must not cost the measurement
        res["bed"] = None
    res["roofline"] = roofline_of(sim, wl, n_now, prof_steps or min(steps, 200))
    res["e2e"] = e2e_of(sim, len(wl["radius"]), steps, dist)
    final = sim.get_state()
    if keep:
        return sim, res, final
    del sim
    return None, res, final


def prepared(rp, wl, log):
    """The workload's relaxed start (radii grown from 0.6x with overlaps
    removed, on the product engine; not timed)."""
    if wl["name"].startswith(("hopper", "adhesive", "batched", "drum")):
        relax(rp, wl, log=log)
    return wl


def jkr_network(rp, wl, state, log):
    """Train the JKR network once on the GPU for a workload; returns the arrays
    set_jkr_network takes and the training report."""
    sim = make_sim(rp, wl_at(wl, state))
    rep = sim.train_jkr_network(seed=1)
    net = sim.get_jkr_network()
    del sim
    log(f"JKR network trained in {rep['train_ms']:.0f} ms (held-out rms {rep['val_rms']:.2e})")
    return net, rep


def form_entry(res, force_err=None, extra=None):
    e = {k: res[k] for k in ("value", "ms_per_step", "particles", "mode", "precision", "clocks", "gpu_launches", "bed",
                             "verlet_skin_m")}
    e["e2e"] = {"value": res["e2e"]["value"], "wall_ms": res["e2e"]["wall_ms"],
                "h2d_bytes_per_step": res["e2e"]["h2d_bytes_per_step"],
                "d2h_bytes_per_step": res["e2e"]["d2h_bytes_per_step"]}
    e["roofline_frac"] = res["roofline"]["frac"]
    e["force_ms"] = res["roofline"]["avg_launch_ms"]
    if "jkr" in res:
        e["jkr"] = res["jkr"]
    if "autotune" in res:
        e["autotune"] = res["autotune"]
    if force_err is not None:
        e["force_err"] = force_err
    if extra:
        e.update(extra)
    return e


def settled_state(rp, wl, mode, precision, jkr, settle, device, log):
    """The state after `settle` untimed steps from the workload's relaxed start."""
    sim = make_sim(rp, wl, mode, precision)
    sim._L.rp_enable_gpu(sim._h, device)
    setup_jkr(sim, jkr)
    t0 = time.time()
    sim.steps(settle)
    st = sim.get_state()
    del sim
    log(f"{wl['name']}: settled {settle} steps in {time.time() - t0:.1f} s")
    return st


def run_forms(rp, args, dist, device, log, headline_state, hopper_wl, cache, threads, deadline):
    """Every spec form beside the plain one, each on its own benchmark
    workload (see the module docstring); each entry carries its own value,
    e2e, roofline fraction, force error against the FP64 oracle and clocks."""
    forms = {}
    K = args.steps

    def budget_ok(name):
        if time.time() < deadline:
            return True
        forms.setdefault("skipped", []).append(f"{name}: time budget of the run used up")
        return False

    def attempt(name, fn):
        if not budget_ok(name):
            return
        try:
            fn()
        except Exception as ex:  # a failing form must not take the headline with it
            forms.setdefault("errors", {})[name] = f"{type(ex).__name__}: {ex}"
            log(f"form {name} failed: {ex}")

    sel = set(args.forms.split(",")) if args.forms else {"hopper", "adhesive", "drum", "batched"}

    def hopper_forms():
        h = forms.setdefault("hopper-1M", {})
        _, r, st = run_form(rp, hopper_wl, args, dist, device, log, precision="mixed", state=headline_state)
        fp = fp64_roofline(rp, hopper_wl, r["particles"], r["ms_per_step"], "-mixed")
        h["mixed"] = form_entry(r, force_error(rp, hopper_wl, headline_state, "parity", "mixed", None, cache, log,
                                               threads), {"fp64_frac": fp.get("frac") if fp else None})
        _, r, st = run_form(rp, hopper_wl, args, dist, device, log, mode="physical", state=headline_state, settle=300)
        h["physical"] = form_entry(r, force_error(rp, hopper_wl, st, "physical", "fp64", None, cache, log, threads),
                                   {"note": "300 untimed steps from the settled parity state load the springs"})

    def adhesive_forms():
        wl = prepared(rp, adhesive_workload(n=int(4_194_304 * args.form_scale)), log)
        a = forms.setdefault("adhesive-4M", {})
        st = settled_state(rp, wl, "parity", "fp64", {"solver": "certified"}, wl["settle"], device, log)
        net, rep = jkr_network(rp, wl, st, log)
        a["training"] = {k: rep[k] for k in ("train_ms", "val_rms", "val_max", "samples", "steps")}
        for name, prec, solver in (("certified", "fp64", "certified"), ("learned", "fp64", "learned"),
                                   ("learned_mixed", "mixed", "learned"), ("newton_mixed", "mixed", "newton"),
                                   ("newton", "fp64", "newton")):
            if not budget_ok(f"adhesive {name}"):
                break
            jk = {"solver": solver, "network": net}
            _, r, _ = run_form(rp, wl, args, dist, device, log, precision=prec, jkr=jk, state=st,
                               prof_steps=min(K, 20))
            a[name] = form_entry(r, force_error(rp, wl, st, "parity", prec, jk, cache, log, threads))
        a["note"] = "every solver from the same settled state (1,600 steps of the certified solver)"

    def drum_forms():
        wl = prepared(rp, drum_workload(n=int(16_777_216 * args.form_scale)), log)
        d = forms.setdefault("drum-16M", {})
        _, r, st = run_form(rp, wl, args, dist, device, log, settle=wl["settle"])
        d["fp64"] = form_entry(r, force_error(rp, wl, st, "parity", "fp64", None, cache, log, threads))
        _, r, _ = run_form(rp, wl, args, dist, device, log, precision="mixed", state=st)
        d["mixed"] = form_entry(r, force_error(rp, wl, st, "parity", "mixed", None, cache, log, threads))
        cache.pop((wl["name"], 0), None)
        cache.pop((wl["name"], 0, "oracle"), None)

    def batched_forms():
        wl = prepared(rp, batched_workload(n_boxes=max(8, int(args.boxes * args.form_scale))), log)
        b = forms.setdefault(wl["name"], {})
        _, r, st = run_form(rp, wl, args, dist, device, log, settle=wl["settle"], autotune=not args.no_autotune)
        b["device_loop"] = form_entry(r, force_error(rp, wl, st, "parity", "fp64", None, cache, log, threads),
                                      {"boxes": int(len(wl["counts"]))})
        b["one_at_a_time"] = one_at_a_time(rp, wl, min(K, 100))

    if "hopper" in sel:
        attempt("hopper", hopper_forms)
    if "adhesive" in sel:
        attempt("adhesive", adhesive_forms)
    if "drum" in sel:
        attempt("drum", drum_forms)
    if "batched" in sel:
        attempt("batched", batched_forms)
    return forms


def cpu_baselines(wl, state, cache, threads, budget_s, log):
    """The reference algorithm on the host cores: (1) on the full settled bed
    with the reference grid's cell at the largest cutoff (the reference's 1 m
    cell makes the candidate search O(N^2) at this size) and the wall loop
    culled exactly, (2) literally (1 m cells, every triangle per particle) on
    the 4,096 particles nearest the bed centre. FP64, OpenMP over particles."""
    from oracle import oracle as om
    om.build()
    om.set_threads(threads)
    n = len(state["radius"])
    hc = max_cutoff(wl)
    o = cache.pop((wl["name"], 0, "oracle"), None)
    if o is None:
        o = oracle_for(wl, state, cell=hc, cull=True)
    rate, k, t = time_oracle(o, n, budget_s * 0.7, max_steps=200)
    del o
    full = {"value": rate, "unit": UNIT, "cores": om.get_threads(), "kind": "port",
            "sample": (f"the full settled bed ({n:,} particles, {len(wl['tri_v']):,} triangles), {k} steps "
                       f"({t:.1f} s) of the reference algorithm in FP64 with the reference grid's cell at the "
                       f"largest cutoff ({hc * 1e3:.4g} mm instead of 1 m) and the every-triangle wall loop culled "
                       "by a triangle grid (same contacts, same order); OpenMP over particles")}
    idx = cpu_sample(dict(wl, position=state["position"]), min(n, 4096))
    lit = oracle_for(wl, state, cell=1.0, cull=False, idx=idx)
    rate2, k2, t2 = time_oracle(lit, len(idx), budget_s * 0.3, max_steps=200)
    del lit
    literal = {"value": rate2, "unit": UNIT, "cores": om.get_threads(), "kind": "port",
               "sample": (f"{len(idx):,} particles nearest the bed centre with all {len(wl['tri_v']):,} triangles, "
                          f"{k2} steps ({t2:.1f} s); the literal reference algorithm (1 m cells, every triangle per "
                          "particle), FP64; its per-particle cost grows with N")}
    log(f"CPU baseline: {rate:.3e} particle-steps/s (full bed), {rate2:.3e} (literal sample)")
    return full, literal


# -------------------------------------------------------------------- arms
def common_config(wl, ws, mode="parity"):
    n = len(wl["radius"])
    return {"workload": wl["name"], "describe": wl["describe"], "particles": int(n), "mode": mode,
            "parallelism": f"replicas x{ws}",
            "l2": f"inputs larger than L2 (particle state {n * 312 / 1e6:.0f} MB)"}


def run_reference(args, log):
    """The reference's CPU step on the host cores (the oracle's restatement in
    f32, the reference's own precision), on the same workload as the GPU arm:
    every particle, K timed steps after W warm-up steps, all host threads."""
    ws, rank, _ = dist_info()
    dist = init_dist(ws)
    if rank != 0:
        barrier(dist)
        return 0
    wl = make_workload(args)
    threads = os.cpu_count() or 1
    from oracle import oracle as om
    om.build()
    om.set_threads(threads)
    hc = max_cutoff(wl)
    o = oracle_for(wl, prec=32, cell=hc, cull=True)
    n = len(wl["radius"])
    o.steps(max(1, args.warmup))
    t0 = time.perf_counter()
    o.steps(args.steps)
    t = time.perf_counter() - t0
    value = n * args.steps / t
    sample = (f"every particle of the workload's seeded start state ({n:,} particles, {len(wl['tri_v']):,} "
              f"triangles), {args.steps} timed steps after {max(1, args.warmup)} warm-up steps; the reference "
              f"algorithm in f32 with the reference grid's cell at the largest cutoff ({hc * 1e3:.4g} mm instead of "
              "1 m, whose candidate search is O(N^2) here) and the every-triangle wall loop culled by a triangle "
              "grid (same contacts, same order); OpenMP over particles")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": common_config(wl, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": om.get_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def run_ours(args, log):
    t_start = time.time()
    ws, rank, local = dist_info()
    dist = init_dist(ws)
    import torch
    import rusty_particles_gb300 as rp
    torch.cuda.set_device(local)
    threads = os.cpu_count() or 1
    wl = make_workload(args)
    loaded = None
    if args.state_in:  # a settled state saved by --state-out (positions, velocities, ...)
        loaded = dict(np.load(args.state_in))
        wl["position"] = loaded["position"]
    else:
        prepared(rp, wl, log)
    jkr = None
    if wl["normal"] == "jkr":
        solver = args.jkr_solver or "learned"
        jkr = {"solver": solver}
        if solver == "learned":
            if args.jkr_net_in:
                z = np.load(args.jkr_net_in)
                jkr["network"] = (z["params"], z["norm"], z["domain"])
            else:
                jkr["network"], _ = jkr_network(rp, wl, {"position": wl["position"], "radius": wl["radius"],
                                                         "mass": wl["mass"]}, log)
            if args.jkr_net_out:
                p, nm, dm = jkr["network"]
                np.savez(args.jkr_net_out, params=p, norm=nm, domain=dm)
    state = None
    settle = 0 if loaded is not None else int(wl.get("settle", 0))
    if loaded is not None:
        state = {k: v for k, v in loaded.items()}
    if args.state_out:
        sim0 = make_sim(rp, wl, args.mode, args.precision)
        setup_jkr(sim0, jkr)
        sim0.steps(settle)
        np.savez(args.state_out, **sim0.get_state())
        del sim0
        settle = 0
        state = dict(np.load(args.state_out))
    if args.profile_only:
        sim = make_sim(rp, wl if state is None else wl_at(wl, state), args.mode, args.precision)
        if args.host_loop:
            sim._L.rp_set_device_loop(sim._h, 0)
        setup_jkr(sim, jkr)
        if state is not None:
            set_dynamic_state(sim, state)
        sim.steps(settle + args.warmup)
        s0, s1, wall, ck = timed(sim, args.steps, dist, local)
        if rank == 0:
            print(json.dumps({"profile_only": True, "particles": int(s1["particles"]), "steps": args.steps,
                              "ms_per_step": (s1["device_ms"] - s0["device_ms"]) / args.steps,
                              "gpu_launches": int(s1["kernel_launches"] - s0["kernel_launches"])}), flush=True)
        return 0
    _, res, final = run_form(rp, wl, args, dist, local, log, mode=args.mode, precision=args.precision, jkr=jkr,
                             state=state, settle=settle, autotune=args.autotune or (
                                 args.workload == "batched" and not args.no_autotune),
                             host_loop=args.host_loop)
    res["roofline"]["traffic"], res["roofline"]["fp64_pipe_active_pct"] = profiled_traffic(wl["name"],
                                                                                           res["particles"])
    res["roofline"]["fp64"] = fp64_roofline(rp, wl, res["particles"], res["ms_per_step"])
    if rank != 0:
        barrier(dist)
        return 0
    cache = {}
    ferr = None
    cpu, cpu_lit = None, None
    if not args.no_force_err:
        try:
            ferr = force_error(rp, wl, final, args.mode, args.precision, jkr, cache, log, threads, keep_oracle=True)
        except Exception as ex:
            ferr = {"error": f"{type(ex).__name__}: {ex}"}
    if not args.no_cpu and "groups" not in wl:
        cpu, cpu_lit = cpu_baselines(wl, final, cache, threads, args.cpu_budget, log)
    forms = None
    if ws == 1 and not args.no_forms and args.workload == "hopper" and args.mode == "parity" \
            and args.precision == "fp64":
        got = run_forms(rp, args, dist, local, log, final, wl, cache, threads, t_start + args.forms_budget)
        plain = form_entry(res, ferr, {"fp64_frac": (res["roofline"].get("fp64") or {}).get("frac")})
        forms = {"hopper-1M": {"plain": plain, **got.pop("hopper-1M", {})}}
        forms.update(got)
    line = {
        "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32-pairs/f64-state",
        "data": "synthetic", "config": common_config(wl, ws, args.mode),
        "roofline": res["roofline"], "cpu_baseline": cpu, "cpu_baseline_literal": cpu_lit,
        "e2e": res["e2e"], "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
        "force_err": ferr, "precision": args.precision, "wall_s_timed": res["wall_s_timed"],
        "stats": res["stats"], "verlet_skin_m": res["verlet_skin_m"], "bed": res.get("bed"),
    }
    if "jkr" in res:
        line["jkr"] = res["jkr"]
    if "autotune" in res:
        line["autotune"] = res["autotune"]
    if args.workload == "batched":
        line["boxes"] = int(len(wl["counts"]))
        line["one_at_a_time"] = one_at_a_time(rp, wl, min(args.steps, 100))
    if forms is not None:
        line["forms"] = forms
    line["bench_wall_s"] = round(time.time() - t_start, 1)
    print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 300 timed steps span a few list rebuilds of the hopper bed (one per ~130
    # steps), so the rebuilds' share of the step is in the headline
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["hopper", "box", "adhesive", "batched", "drum"], default="hopper")
    ap.add_argument("--boxes", type=int, default=512, help="boxes of the batched workload")
    ap.add_argument("--autotune", action="store_true", help="autotune launch shapes before timing")
    ap.add_argument("--no-autotune", action="store_true", help="batched workload: keep default launch shapes")
    ap.add_argument("--jkr-solver", choices=["newton", "learned", "certified"], default=None,
                    help="JKR solver of the adhesive workload (default learned)")
    ap.add_argument("--jkr-net-in", default=None, help="trained JKR network (.npz) instead of training")
    ap.add_argument("--jkr-net-out", default=None, help="save the trained JKR network (.npz)")
    ap.add_argument("--mode", choices=["parity", "physical"], default="parity")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines")
    ap.add_argument("--no-force-err", action="store_true", help="skip the force error against the oracle")
    ap.add_argument("--no-forms", action="store_true", help="skip the other forms (headline hopper run only)")
    ap.add_argument("--forms", default=None, help="comma list of form workloads: hopper,adhesive,drum,batched")
    ap.add_argument("--forms-budget", type=float, default=600.0,
                    help="seconds from the start after which no further form starts")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--form-scale", type=float, default=1.0,
                    help="scale of the other forms' workloads (1 = the benchmark sizes; smaller for quick checks)")
    ap.add_argument("--particles", type=int, default=None,
                    help="workload size (hopper 1,048,576, adhesive 4,194,304 by default)")
    ap.add_argument("--state-in", default=None, help="settled state (.npz from --state-out) instead of relaxing")
    ap.add_argument("--state-out", default=None, help="save the settled state (.npz) before the warm-up")
    ap.add_argument("--host-loop", action="store_true", help="host-issued kernels instead of the device loop")
    ap.add_argument("--skin", type=float, default=None,
                    help="Verlet skin in m for the timed simulations (default: 0.2 of the largest radius)")
    ap.add_argument("--profile-only", action="store_true", help="warm-up + timed steps only (for ncu)")
    args = ap.parse_args()
    log = (lambda m: print(m, file=sys.stderr, flush=True))
    if args.impl == "reference":
        return run_reference(args, log)
    return run_ours(args, log)


if __name__ == "__main__":
    sys.exit(main())
