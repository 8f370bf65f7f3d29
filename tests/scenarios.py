"""The reference's integration scenarios, written once and run against any
object with the reference's `Simulation` surface (src/lib.rs:41-277).

Each function restates the setup, stepping and assertion of one test in the
reference's `pydem/` directory (cited per function) and returns the measured
quantity. The CPU suite runs them against the oracle; the GPU suite runs them
against the product module `rusty_particles_gb300`.
"""
import math
import os
import random

import numpy as np

from tests.stl_util import floor_tris, write_binary_stl


def free_fall(create):
    """pydem/test_analytical.py:13-48 — y(t) = y0 - g t^2/2 within 1e-2."""
    dt, total, g, y0 = 1e-6, 1.0, 9.81, 10.0
    sim = create(dt, -10.0, 0.0, -10.0, 10.0, 20.0, 10.0, 10)
    sim.add_particle(0.0, y0, 0.0, 0.1, 1.0)
    sim.run(total)
    _, y, _ = sim.get_particle_position(0)
    err = abs(y - (y0 - 0.5 * g * total ** 2))
    assert err < 1e-2, err
    return err


def hertzian_compression(create):
    """pydem/test_analytical.py:51-112 — static Hertz overlap within 1e-5 absolute."""
    dt, total, g, radius, mass, E, nu = 1e-4, 1.0, 9.81, 0.1, 1.0, 1e7, 0.3
    sim = create(dt, -1.0, -1.0, -1.0, 1.0, 2.0, 1.0, 10)
    sim.set_particle_material(E, nu, 2500.0, 0.5, 0.5)
    sim.add_particle(0.0, 0.0, 0.0, radius, 1e9, fixed=True)
    sim.add_particle(0.0, 2.0 * radius, 0.0, radius, mass)
    sim.run(total)
    _, y1, _ = sim.get_particle_position(0)
    _, y2, _ = sim.get_particle_position(1)
    overlap = 2.0 * radius - (y2 - y1)
    r_star = radius / 2.0
    e_star = E / (2.0 * (1.0 - nu ** 2))
    expect = ((3.0 * mass * g) / (4.0 * e_star * np.sqrt(r_star))) ** (2.0 / 3.0)
    err = abs(overlap - expect)
    assert err < 1e-5, err
    return err


def rolling(create, workdir):
    """pydem/test_analytical_rotation.py:13-169 — time to pure rolling 2v0/(7 mu g) within 5 %.

    The ball starts on the shared diagonal edge of the two floor triangles, so
    it touches both (a double contact), as in the reference test.
    """
    radius, mass, v0, mu, g, dt = 0.05, 1.0, 1.0, 0.1, 9.81, 1e-4
    expected = (2 * v0) / (7 * mu * g)
    sim = create(dt, -10.0, 0.0, -10.0, 10.0, 10.0, 10.0, 1)
    sim.set_particle_material(1e8, 0.3, 2500.0, mu, 0.5)
    sim.set_wall_material(1e8, 0.3, 2500.0, mu, 0.5)
    sim.set_contact_models("Hertzian", "Coulomb")
    path = os.path.join(workdir, "floor.stl")
    write_binary_stl(path, floor_tris())
    sim.add_mesh(path)
    sim.add_particle(0.0, radius, 0.0, radius, mass)
    sim.set_particle_velocity(0, v0, 0.0, 0.0)
    t = 0.0
    for _ in range(10000):
        sim.step()
        t += dt
        vx, _, _ = sim.get_particle_velocity(0)
        _, _, wz = sim.get_particle_angular_velocity(0)
        if vx + wz * radius <= 0.0:
            break
    else:
        raise AssertionError("did not reach pure rolling within 10000 steps")
    err = abs(t - expected) / expected
    assert err < 0.05, (t, expected)
    return err


def jkr_pull_off(create):
    """pydem/test_jkr.py:11-90 — minimum force equals -(2/3) pi gamma R* within 10 %."""
    radius, mass, gamma, E, nu = 0.005, 1.0, 0.1, 1e7, 0.3
    r_star = radius / 2.0
    expected = -(2.0 / 3.0) * np.pi * gamma * r_star
    e_star = 1.0 / (2.0 * (1.0 - nu ** 2) / E)
    a_eq = (9.0 * np.pi * gamma * r_star ** 2 / (2.0 * e_star)) ** (1.0 / 3.0)
    delta_eq = a_eq ** 2 / r_star - np.sqrt(8.0 * np.pi * gamma * a_eq / e_star)
    dt = 1e-5
    sim = create(dt, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 2)
    sim.set_particle_material(E, nu, 2500.0, 0.5, 0.5, gamma)
    sim.set_contact_models("JKR", "Coulomb")
    sim.add_particle(0.0, 0.0, 0.0, radius, mass, True)
    sim.add_particle(2.0 * radius - delta_eq, 0.0, 0.0, radius, mass, False)
    sim.set_particle_velocity(1, 0.002, 0.0, 0.0)
    fmin = 0.0
    for _ in range(50000):
        vp, _, _ = sim.get_particle_velocity(1)
        sim.step()
        vc, _, _ = sim.get_particle_velocity(1)
        f = mass * (vc - vp) / dt
        fmin = min(fmin, f)
        x, _, _ = sim.get_particle_position(1)
        if 2.0 * radius - x < -radius:
            break
    err = abs(fmin - expected) / abs(expected)
    assert err < 0.1, (fmin, expected)
    return err


def sjkr_pull_off(create):
    """pydem/test_sjkr.py:12-109 — |minimum force| equals 1.5 pi gamma R* within 10 %."""
    radius, mass, gamma, E, nu = 0.005, 1.0, 0.5, 1e5, 0.3
    r_star = radius / 2.0
    expected = 1.5 * np.pi * gamma * r_star
    e_star = 1.0 / (2.0 * (1.0 - nu ** 2) / E)
    delta_c = -np.sqrt(3.0 * np.pi ** 2 * gamma ** 2 * r_star / e_star ** 2)
    dt = 1e-5
    sim = create(dt, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 2)
    sim.set_particle_material(E, nu, 2500.0, 0.5, 0.5, gamma)
    sim.set_contact_models("sJKR", "Coulomb")
    sim.add_particle(0.0, 0.0, 0.0, radius, mass, True)
    sim.add_particle(2.0 * radius - radius * 0.01, 0.0, 0.0, radius, mass, False)
    sim.step()
    vp, _, _ = sim.get_particle_velocity(1)
    sim.step()
    vc, _, _ = sim.get_particle_velocity(1)
    sim.set_particle_velocity(1, 0.01, 0.0, 0.0)
    fmin = 0.0
    for _ in range(50000):
        vp, _, _ = sim.get_particle_velocity(1)
        sim.step()
        vc, _, _ = sim.get_particle_velocity(1)
        fmin = min(fmin, mass * (vc - vp) / dt)
        x, _, _ = sim.get_particle_position(1)
        if 2.0 * radius - x < delta_c * 1.1:
            break
    err = abs(abs(fmin) - expected) / expected
    assert err < 0.1, (fmin, expected)
    return err


def contact_models(create, raises):
    """pydem/test_models.py:12-33 — valid names accepted, invalid raises ValueError, empty runs."""
    sim = create(0.001, -1.0, 0.0, -1.0, 1.0, 5.0, 1.0, 100)
    sim.run(0.1)
    sim.set_contact_models("linear", "coulomb")
    sim.run(0.1)
    for n in ["hertz", "Hertzian", "LINEAR", "spring_dashpot", "hysteretic", "jkr", "sjkr", "simplified_jkr"]:
        for t in ["mindlin", "Coulomb", "linear", "spring_coulomb"]:
            sim.set_contact_models(n, t)
    with raises(ValueError):
        sim.set_contact_models("invalid", "coulomb")
    with raises(ValueError):
        sim.set_contact_models("hertz", "invalid")
    return sim.get_particle_count()


def periodic_y(create, seed=1234):
    """pydem/test_periodic.py:12-47 — 101 particles, y periodic, 100 steps (seeded here)."""
    rng = random.Random(seed)
    sim = create(0.01, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 1)
    sim.set_periodic_boundary(False, True, False)
    sim.add_particle(0.9, 0.0, 0.0, 0.1, 1.0)
    sim.set_periodic_boundary(False, True, False)
    for _ in range(100):
        x = rng.uniform(-0.4, 0.4)
        z = rng.uniform(-0.4, 0.4)
        y = rng.uniform(1.0, 4.0)
        sim.add_particle(x, y, z, rng.uniform(0.02, 0.03), 1.0)
    for _ in range(100):
        sim.step()
    return sim


def column_1000(create):
    """pydem/test_multithreading.py:12-34 — 1000 heavily overlapping particles, run(0.1)."""
    sim = create(0.001, -1.0, 0.0, -1.0, 1.0, 5.0, 1.0, 5000)
    for i in range(1000):
        sim.add_particle(0.0, 2.0 + i * 0.001, 0.0, 0.05, 1.0)
    sim.run(0.1)
    return sim


def triangle_known_answer(query):
    """src/mesh.rs:150-172 — penetration 0.1 and normal +Z within 1e-5; far sphere misses."""
    tri = [0, 0, 0, 1, 0, 0, 0, 1, 0]
    nrm = [0, 0, 1]
    hit = query(tri, nrm, [0.2, 0.2, 0.5], 0.6)
    assert hit is not None
    pen, n = hit
    assert abs(pen - 0.1) < 1e-5
    assert np.linalg.norm(np.asarray(n) - np.array([0, 0, 1.0])) < 1e-5
    assert query(tri, nrm, [0.2, 0.2, 2.0], 0.5) is None
    return pen
