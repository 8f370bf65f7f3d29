"""rusty_particles_gb300 — the rusty_particles DEM step on GB300 (sm_103a).

A drop-in for the reference's Python module ``rusty_particles``
(src/lib.rs:24-35)::

    import rusty_particles_gb300 as rusty_particles
    sim = rusty_particles.Simulation.create(dt, -1, -1, -1, 1, 1, 1, 1000)

Same class, method names, argument order, defaults and exception types as
the reference's pyo3 class (src/lib.rs:41-277). Every step runs on the GPU
through librp.so (include/rp.h); there is no CPU path, so without a CUDA
device stepping raises RuntimeError. Differences from the reference that a
caller can see are listed in the method docstrings (getters read current GPU
state; `enable_gpu` is optional; friction must be >= 0).
"""
from __future__ import annotations

import ctypes
import math
import sys

import numpy as np

from . import _lib
from ._lib import RP_MODE_PARITY, RP_MODE_PHYSICAL, RP_PREC_FP64, RP_PREC_MIXED, RpState, RpStats, check

__all__ = ["Simulation", "set_num_threads", "hello", "RP_PREC_FP64", "RP_PREC_MIXED", "RP_MODE_PARITY",
           "RP_MODE_PHYSICAL"]

_OVERLAP_WARNING = "Warning: Excessive particle overlap detected (>20% of radius). Simulation may be unstable."


def set_num_threads(num_threads):
    """src/lib.rs:15-22: sizes the host thread pool once; a second call raises RuntimeError."""
    check(_lib.load().rp_set_threads(int(num_threads)))


def hello():
    """src/lib.rs:29-32."""
    return "Hello from rusty_particles_gb300!"


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Simulation:
    """The reference's `Simulation` (src/lib.rs:41-277) on a GB300."""

    def __init__(self, handle, dt):
        self._L = _lib.load()
        self._h = handle
        self._dt = float(dt)
        self._warned = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.rp_destroy(h)
            self._h = None

    # ---- src/lib.rs:57 ----------------------------------------------------
    @staticmethod
    def create(dt, min_x, min_y, min_z, max_x, max_y, max_z, particle_count):
        L = _lib.load()
        mn = (ctypes.c_double * 3)(min_x, min_y, min_z)
        mx = (ctypes.c_double * 3)(max_x, max_y, max_z)
        h = L.rp_create(float(dt), mn, mx, int(particle_count))
        if not h:
            raise ValueError(_lib.last_error())
        return Simulation(h, dt)

    def add_particle(self, x, y, z, radius, mass, fixed=False):
        """src/lib.rs:76-80."""
        check(self._L.rp_add_particle(self._h, x, y, z, radius, mass, 1 if fixed else 0))

    def add_particles(self, positions, radii, masses, fixed=None):
        """Bulk add (no reference counterpart): positions [N,3], radii [N], masses [N]."""
        pos = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(radii, np.float64).reshape(-1)
        m = np.ascontiguousarray(masses, np.float64).reshape(-1)
        fx = None
        if fixed is not None:
            fx = np.ascontiguousarray(fixed, np.uint8).reshape(-1)
        check(self._L.rp_add_particles(self._h, len(pos), _dptr(pos), _dptr(r), _dptr(m),
                                       fx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if fx is not None else None))

    def add_mesh(self, path):
        """src/lib.rs:87-91: binary or ASCII STL; IOError on failure."""
        check(self._L.rp_add_mesh_stl(self._h, str(path).encode()))

    def add_triangles(self, vertices, normals=None, group=None, motion=None):
        """Triangles as a [T,9] array (no reference counterpart); `group`
        restricts them to the particles of one group; `motion` = (center,
        omega, velocity) gives their surface the velocity
        velocity + omega x (p - center) (the geometry stays put)."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
        n = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        fp = ctypes.POINTER(ctypes.c_float)
        nptr = n.ctypes.data_as(fp) if n is not None else None
        if motion is not None:
            c, w, u = (np.ascontiguousarray(a, np.float64).reshape(3) for a in motion)
            g = _lib.RP_GROUP_ALL if group is None else int(group)
            check(self._L.rp_add_mesh_triangles_moving(self._h, len(v), v.ctypes.data_as(fp), nptr, g, _dptr(c),
                                                       _dptr(w), _dptr(u)))
        elif group is None:
            check(self._L.rp_add_mesh_triangles(self._h, len(v), v.ctypes.data_as(fp), nptr))
        else:
            check(self._L.rp_add_mesh_triangles_group(self._h, len(v), v.ctypes.data_as(fp), nptr, int(group)))

    # ---- launch shapes ------------------------------------------------------
    def autotune(self):
        """Choose the force pass's launch shapes on the current state (after a step)."""
        r = _lib.RpTuneReport()
        check(self._L.rp_autotune(self._h, ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in _lib.RpTuneReport._fields_}

    def set_launch_shape(self, bs_filter=0, bs_force=0, bs_accum=0, grid_cap=0):
        check(self._L.rp_set_launch_shape(self._h, int(bs_filter), int(bs_force), int(bs_accum), int(grid_cap)))

    # ---- groups: independent beds in one simulation -----------------------
    def set_particle_groups(self, groups):
        g = np.ascontiguousarray(groups, np.uint32)
        check(self._L.rp_set_particle_groups(self._h, g.size, g.ctypes.data_as(_lib._u32p)))

    def get_particle_groups(self):
        g = np.zeros(self.get_particle_count(), np.uint32)
        check(self._L.rp_get_particle_groups(self._h, g.size, g.ctypes.data_as(_lib._u32p)))
        return g

    def set_group_material(self, group, youngs_modulus, poissons_ratio, density, friction_coefficient,
                           restitution_coefficient, surface_energy):
        check(self._L.rp_set_group_material(self._h, int(group), youngs_modulus, poissons_ratio, density,
                                            friction_coefficient, restitution_coefficient, surface_energy))

    def step(self):
        """src/lib.rs:94."""
        check(self._L.rp_step(self._h, 1))
        self._warn()

    def steps(self, n):
        """n steps in one call (no reference counterpart)."""
        check(self._L.rp_step(self._h, int(n)))
        self._warn()

    def set_particle_material(self, youngs_modulus, poissons_ratio, density, friction_coefficient,
                              restitution_coefficient, surface_energy=0.0):
        """src/lib.rs:98-109 (friction before restitution, as the reference's signature)."""
        check(self._L.rp_set_particle_material(self._h, youngs_modulus, poissons_ratio, density,
                                               friction_coefficient, restitution_coefficient, surface_energy))

    def set_wall_material(self, youngs_modulus, poissons_ratio, density, friction_coefficient,
                          restitution_coefficient, surface_energy=0.0):
        """src/lib.rs:126-129."""
        check(self._L.rp_set_wall_material(self._h, youngs_modulus, poissons_ratio, density,
                                           friction_coefficient, restitution_coefficient, surface_energy))

    def set_periodic_boundary(self, x, y, z):
        """src/lib.rs:138."""
        check(self._L.rp_set_periodic(self._h, int(bool(x)), int(bool(y)), int(bool(z))))

    def enable_gpu(self):
        """src/lib.rs:146-148: initialises the CUDA device and uploads the particles.

        Stepping always runs on the GPU, so calling this is optional; it raises
        RuntimeError when no CUDA device is usable.
        """
        check(self._L.rp_enable_gpu(self._h, -1))

    def init_mpi(self):
        """src/lib.rs:150: with one process the reference's slab is the whole box, so this is a no-op."""
        return None

    def set_contact_models(self, normal, tangential):
        """src/lib.rs:160-180: case-insensitive names; ValueError for unknown ones."""
        nm, tm = ctypes.c_int(), ctypes.c_int()
        check(self._L.rp_parse_contact_models(str(normal).encode(), str(tangential).encode(), ctypes.byref(nm),
                                              ctypes.byref(tm)))
        check(self._L.rp_set_contact_models(self._h, nm.value, tm.value))

    def run(self, duration):
        """src/lib.rs:182-195: ceil(duration / dt) steps, computed in f32."""
        check(self._L.rp_run(self._h, float(duration)))
        self._warn()

    def write_vtk(self, filename):
        """src/lib.rs:202-207 / src/vtk.rs:5-44; IOError on failure."""
        check(self._L.rp_write_vtk(self._h, str(filename).encode()))

    def get_particle_count(self):
        return int(self._L.rp_particle_count(self._h))

    def _get(self, fn, i):
        if i < 0:
            raise IndexError("Particle index out of bounds")
        out = (ctypes.c_double * 3)()
        check(fn(self._h, int(i), out))
        return (out[0], out[1], out[2])

    def get_particle_position(self, id):
        """src/lib.rs:223-230. Reads the current device state (the reference's
        GPU mode returns values stale since enable_gpu)."""
        return self._get(self._L.rp_get_particle_position, id)

    def get_particle_velocity(self, id):
        return self._get(self._L.rp_get_particle_velocity, id)

    def get_particle_angular_velocity(self, index):
        return self._get(self._L.rp_get_particle_angular_velocity, index)

    def set_particle_velocity(self, id, vx, vy, vz):
        if id < 0:
            raise IndexError("Particle index out of bounds")
        check(self._L.rp_set_particle_velocity(self._h, int(id), vx, vy, vz))

    def set_particle_angular_velocity(self, index, x, y, z):
        if index < 0:
            raise IndexError("Particle index out of bounds")
        check(self._L.rp_set_particle_angular_velocity(self._h, int(index), x, y, z))

    # ---- extensions -------------------------------------------------------
    def set_precision(self, precision):
        """RP_PREC_FP64 (default) or RP_PREC_MIXED (FP32 pair math, FP64 state)."""
        p = {"fp64": RP_PREC_FP64, "mixed": RP_PREC_MIXED}.get(precision, precision)
        check(self._L.rp_set_precision(self._h, int(p)))

    def set_interaction_mode(self, mode):
        """RP_MODE_PARITY (default; the reference's rules) or RP_MODE_PHYSICAL."""
        m = {"parity": RP_MODE_PARITY, "physical": RP_MODE_PHYSICAL}.get(mode, mode)
        check(self._L.rp_set_interaction_mode(self._h, int(m)))

    def set_gravity(self, gx, gy, gz):
        check(self._L.rp_set_gravity(self._h, gx, gy, gz))

    def set_skin(self, skin):
        check(self._L.rp_set_skin(self._h, float(skin)))

    def set_neighbor_capacity(self, cap):
        check(self._L.rp_set_neighbor_capacity(self._h, int(cap)))

    def set_reference_cell_size(self, h):
        check(self._L.rp_set_reference_cell_size(self._h, float(h)))

    def set_debug(self, on=True):
        check(self._L.rp_set_debug(self._h, 1 if on else 0))

    def stats(self):
        s = RpStats()
        check(self._L.rp_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in RpStats._fields_}

    def bed_statistics(self):
        """Kinetic energy, coordination number (2 x overlapping pairs / N) and
        solid fraction of the box of the current state, computed on the GPU
        (needs one completed step)."""
        out = (ctypes.c_double * 3)()
        check(self._L.rp_bed_statistics(self._h, out))
        return {"kinetic_energy": out[0], "coordination_number": out[1], "solid_fraction_box": out[2]}

    def get_state(self, out=None):
        """All per-particle state as numpy arrays in id order. `out` (a dict as
        returned here, e.g. from an earlier call) is filled in place instead of
        allocating: its arrays must be C-contiguous float64 (uint8 for
        `fixed`) of the current particle count; keys it lacks are skipped."""
        n = self.get_particle_count()
        if out is not None:
            shapes = {"radius": (n,), "mass": (n,), "fixed": (n,)}
            known = {f for f, _ in RpState._fields_} - {"n_particles"}
            for k, a in out.items():
                if k not in known:
                    raise KeyError(f"unknown state array {k!r}")
                want = np.uint8 if k == "fixed" else np.float64
                if (not isinstance(a, np.ndarray) or a.dtype != want or not a.flags.c_contiguous
                        or a.shape != shapes.get(k, (n, 3)) or not a.flags.writeable):
                    raise ValueError(f"out[{k!r}] must be a writable C-contiguous {np.dtype(want).name} array "
                                     f"of shape {shapes.get(k, (n, 3))}")
            arrs = out
        else:
            arrs = {k: np.zeros((n, 3)) for k in ("position", "velocity", "angular_velocity", "acceleration",
                                                  "torque", "position_residual", "velocity_residual",
                                                  "angular_velocity_residual")}
            arrs["radius"] = np.zeros(n)
            arrs["mass"] = np.zeros(n)
            arrs["fixed"] = np.zeros(n, np.uint8)
        st = RpState()
        st.n_particles = n
        for k, a in arrs.items():
            if k == "fixed":
                st.fixed = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            else:
                setattr(st, k, _dptr(a))
        if n:
            check(self._L.rp_read_state(self._h, ctypes.byref(st)))
        return arrs

    def set_state(self, arrs):
        """Overwrite per-particle state (keys as in get_state; missing keys are
        kept). Every array must hold one entry per current particle: shape
        (n, 3) for vectors and (n,) for radius, mass and fixed, with n =
        get_particle_count(); ValueError otherwise."""
        n = self.get_particle_count()
        known = {f for f, _ in RpState._fields_} - {"n_particles"}
        for k in arrs:
            if k not in known:
                raise KeyError(f"unknown state array {k!r}")
        keep = []
        st = RpState()
        st.n_particles = n
        for k, _ in RpState._fields_:
            if k == "n_particles" or k not in arrs:
                continue
            want = (n,) if k in ("radius", "mass", "fixed") else (n, 3)
            a = np.ascontiguousarray(arrs[k], np.uint8 if k == "fixed" else np.float64)
            if a.shape != want:
                raise ValueError(f"state array {k!r} has shape {a.shape}, expected {want} for {n} particles")
            if k == "fixed":
                st.fixed = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            else:
                setattr(st, k, _dptr(a))
            keep.append(a)
        check(self._L.rp_write_state(self._h, ctypes.byref(st)))

    def debug_forces(self):
        n = self.get_particle_count()
        F = np.zeros((n, 3))
        T = np.zeros((n, 3))
        check(self._L.rp_debug_last_forces(self._h, _dptr(F), _dptr(T)))
        return F, T

    def debug_pairs(self):
        cnt = ctypes.c_size_t()
        check(self._L.rp_debug_contact_pairs(self._h, None, None, None, 0, ctypes.byref(cnt)))
        k = cnt.value
        pi = np.zeros(max(k, 1), np.int64)
        pj = np.zeros(max(k, 1), np.int64)
        vv = np.zeros(max(k, 1), np.int32)
        check(self._L.rp_debug_contact_pairs(self._h, pi.ctypes.data_as(_lib._i64p), pj.ctypes.data_as(_lib._i64p),
                                             vv.ctypes.data_as(_lib._i32p), k, ctypes.byref(cnt)))
        return pi[:k], pj[:k], vv[:k]

    def debug_reference_grid(self, h=1.0):
        n = self.get_particle_count()
        cell = np.zeros(max(n, 1), np.int64)
        order = np.zeros(max(n, 1), np.int64)
        no = ctypes.c_size_t()
        dims = (ctypes.c_int32 * 3)()
        check(self._L.rp_debug_reference_grid(self._h, float(h), cell.ctypes.data_as(_lib._i64p),
                                              order.ctypes.data_as(_lib._i64p), ctypes.byref(no), dims))
        return tuple(dims), cell[:n], order[:no.value]

    # ---- learned JKR contact radius ---------------------------------------
    def train_jkr_network(self, **options):
        """Generate Newton-solved samples and train the JKR network on the GPU.

        Keyword options are the fields of ``rp_jkr_train_options`` (rs_min,
        rs_max, es_scale, gamma_scale, x_min, x_max, seed, samples, epochs,
        batch, lr0, lr1, qat_from_epoch); returns the training report as a dict.
        """
        o = _lib.RpJkrTrainOptions()
        for k, v in options.items():
            if k not in dict(_lib.RpJkrTrainOptions._fields_):
                raise TypeError(f"unknown option {k!r}")
            setattr(o, k, v)
        r = _lib.RpJkrTrainReport()
        check(self._L.rp_jkr_train(self._h, ctypes.byref(o), ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in _lib.RpJkrTrainReport._fields_}

    def set_jkr_solver(self, solver):
        """'newton' (the reference's iteration), 'learned' or 'certified' (no network)."""
        s = {"newton": _lib.RP_JKR_NEWTON, "learned": _lib.RP_JKR_LEARNED,
             "certified": _lib.RP_JKR_CERTIFIED}.get(solver, solver)
        check(self._L.rp_set_jkr_solver(self._h, int(s)))

    def get_jkr_network(self):
        """(params[8705], norm[10], domain[8]) of the installed network, float32."""
        p = np.zeros(_lib.RP_MLP_PARAMS, np.float32)
        nm = np.zeros(10, np.float32)
        dm = np.zeros(8, np.float32)
        check(self._L.rp_jkr_get_network(self._h, p.ctypes.data_as(_lib._fp), nm.ctypes.data_as(_lib._fp),
                                         dm.ctypes.data_as(_lib._fp)))
        return p, nm, dm

    def set_jkr_network(self, params, norm, domain):
        p = np.ascontiguousarray(params, np.float32)
        nm = np.ascontiguousarray(norm, np.float32)
        dm = np.ascontiguousarray(domain, np.float32)
        if p.size != _lib.RP_MLP_PARAMS or nm.size != 10 or dm.size != 8:
            raise ValueError("network needs 8705 parameters, 10 normalisation and 8 domain values")
        check(self._L.rp_jkr_set_network(self._h, p.ctypes.data_as(_lib._fp), nm.ctypes.data_as(_lib._fp),
                                         dm.ctypes.data_as(_lib._fp)))

    def jkr_counters(self):
        out = (ctypes.c_uint64 * 6)()
        check(self._L.rp_jkr_counters(self._h, out))
        return dict(zip(("accepted", "zero", "fallback", "network_rows", "fp32_newton_steps", "walk"), list(out)))

    def _warn(self):
        """The reference prints a warning on every step with an overlap above
        20 % of a radius (src/simulation.rs:528-530); here once per call."""
        try:
            s = RpStats()
            if self._L.rp_get_stats(self._h, ctypes.byref(s)) == 0 and s.overlap_warn_steps > self._warned:
                print(_OVERLAP_WARNING, file=sys.stderr)
                self._warned = s.overlap_warn_steps
        except Exception:
            pass
