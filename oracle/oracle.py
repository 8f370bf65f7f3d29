"""Python face of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a C++ restatement of the reference's CPU step
(src/simulation.rs:173-562 and the modules it calls); see oracle.cpp. This
module loads ``oracle/_build/liboracle.so`` with ctypes and wraps it in a class
with the reference's Python surface (src/lib.rs:41-277), so the reference's
own integration tests can be re-run against it. Only the test suite, the smoke
check and the CPU-baseline leg of the benchmark use it; the product library
never imports it.
"""
from __future__ import annotations

import ctypes
import math
import os
import struct
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

# Model ids follow the reference enum order (src/physics.rs:6-28).
NORMAL_MODELS = {
    "hertz": 1, "hertzian": 1,
    "linear": 0, "spring_dashpot": 0,
    "hysteretic": 2,
    "jkr": 3,
    "sjkr": 4, "simplified_jkr": 4,
}
TANGENTIAL_MODELS = {"mindlin": 2, "coulomb": 0, "linear": 1, "spring_coulomb": 1}
MODE_PARITY, MODE_PHYSICAL = 0, 1


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (g++ and OpenMP)."""
    r = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, d, i, l = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_long
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_long)
        ip = ctypes.POINTER(ctypes.c_int)
        sig = {
            "orc_create": (vp, [i, d, dp, dp]),
            "orc_destroy": (None, [vp]),
            "orc_set_threads": (None, [i]),
            "orc_get_threads": (i, []),
            "orc_add_particle": (None, [vp, d, d, d, d, d, i]),
            "orc_add_triangles": (None, [vp, dp, dp, l]),
            "orc_add_particles": (None, [vp, l, dp, dp, dp, ctypes.POINTER(ctypes.c_ubyte)]),
            "orc_set_wall_cull": (None, [vp, i]),
            "orc_add_triangles_moving": (None, [vp, dp, dp, l, dp]),
            "orc_set_material": (None, [vp, i, d, d, d, d, d, d]),
            "orc_set_models": (None, [vp, i, i]),
            "orc_set_periodic": (None, [vp, i, i, i]),
            "orc_set_mode": (None, [vp, i]),
            "orc_set_cell_size": (None, [vp, d]),
            "orc_set_gravity": (None, [vp, d, d, d]),
            "orc_set_options": (None, [vp, i, i, i]),
            "orc_step": (None, [vp, l]),
            "orc_count": (l, [vp]),
            "orc_overlap_warnings": (l, [vp]),
            "orc_contact_map_size": (l, [vp]),
            "orc_get_vec": (None, [vp, i, dp]),
            "orc_set_vec": (None, [vp, i, dp]),
            "orc_get_scalar": (None, [vp, i, dp]),
            "orc_last_forces": (None, [vp, dp, dp]),
            "orc_last_force_scale": (None, [vp, dp, dp]),
            "orc_grid_dims": (None, [vp, ip]),
            "orc_grid_items": (l, [vp, lp, lp]),
            "orc_grid_now": (i, [vp]),
            "orc_pair_count": (l, [vp]),
            "orc_pairs": (None, [vp, lp, lp]),
            "orc_triangle_query": (i, [i, dp, dp, dp, d, dp, dp]),
            "orc_jkr_force": (d, [d, d, d, d]),
            "orc_jkr_radius": (d, [d, d, d, d, ip]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _lp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_long))


def read_stl(path: str):
    """Read an STL file the way stl_io 0.7.0 exposes it to src/mesh.rs:125-143.

    ASCII files start with ``solid`` followed by ``facet``/``endsolid``
    records; anything else is read as binary (80-byte header, u32 count,
    50-byte records of normal + three vertices as little-endian f32).
    Returns (vertices [T,9] float64 holding the f32 values, normals [T,3]).
    """
    with open(path, "rb") as f:
        data = f.read()
    head = data[:512].lstrip()
    if head[:5].lower() == b"solid":
        toks = data.split()
        if len(toks) > 2 and (b"facet" in toks[:64] or b"endsolid" in toks[:4]):
            return _read_ascii_stl(data)
    if len(data) < 84:
        raise IOError("STL file too short")
    (n,) = struct.unpack_from("<I", data, 80)
    if len(data) < 84 + 50 * n:
        raise IOError("binary STL truncated")
    rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("attr", "<u2")]), count=n, offset=84)
    return rec["v"].astype(np.float64), rec["n"].astype(np.float64)


def _read_ascii_stl(data: bytes):
    toks = data.split()
    verts, norms = [], []
    k = 0
    while k < len(toks):
        if toks[k] == b"facet" and toks[k + 1] == b"normal":
            nrm = [float(np.float32(float(t))) for t in toks[k + 2:k + 5]]
            k += 5
            tri = []
            while len(tri) < 3 and k < len(toks):
                if toks[k] == b"vertex":
                    tri.append([float(np.float32(float(t))) for t in toks[k + 1:k + 4]])
                    k += 4
                else:
                    k += 1
            if len(tri) != 3:
                raise IOError("malformed ASCII STL facet")
            verts.append(sum(tri, []))
            norms.append(nrm)
        else:
            k += 1
    return np.asarray(verts, np.float64).reshape(-1, 9), np.asarray(norms, np.float64).reshape(-1, 3)


class OracleSimulation:
    """The oracle behind the reference's `Simulation` surface (src/lib.rs:41-277)."""

    def __init__(self, dt, mn, mx, prec=64):
        self._L = lib()
        self.prec = prec
        self.dt = float(dt)
        mnv = np.asarray(mn, np.float64)
        mxv = np.asarray(mx, np.float64)
        self._h = self._L.orc_create(prec, self.dt, _dp(mnv), _dp(mxv))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_destroy(h)
            self._h = None

    # --- reference API -------------------------------------------------
    @staticmethod
    def create(dt, min_x, min_y, min_z, max_x, max_y, max_z, particle_count, prec=64):
        return OracleSimulation(dt, (min_x, min_y, min_z), (max_x, max_y, max_z), prec)

    def add_particle(self, x, y, z, radius, mass, fixed=False):
        self._L.orc_add_particle(self._h, x, y, z, radius, mass, 1 if fixed else 0)

    def add_particles(self, xyz, r, m, fixed=None):
        """Bulk add: positions [N,3], radii [N], masses [N], fixed flags [N] (optional)."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        m = np.ascontiguousarray(m, np.float64).reshape(-1)
        fx = None
        if fixed is not None:
            fx = np.ascontiguousarray(fixed, np.uint8).reshape(-1)
        self._L.orc_add_particles(self._h, len(xyz), _dp(xyz), _dp(r), _dp(m),
                                  fx.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) if fx is not None else None)

    def set_wall_cull(self, on=True):
        """Cull the wall loop by a triangle grid: the contacts and their order
        are those of the reference's every-triangle loop (a baseline variant)."""
        self._L.orc_set_wall_cull(self._h, 1 if on else 0)

    def add_mesh(self, path):
        v, n = read_stl(path)
        self.add_triangles(v, n)

    def add_triangles(self, v, n, motion=None):
        """motion = (center, omega, velocity): the surface moves with
        velocity + omega x (p - center) (an extension; None = static walls)."""
        v = np.ascontiguousarray(v, np.float64).reshape(-1, 9)
        n = np.ascontiguousarray(n, np.float64).reshape(-1, 3)
        if motion is None:
            self._L.orc_add_triangles(self._h, _dp(v), _dp(n), len(v))
        else:
            c9 = np.ascontiguousarray(np.concatenate([np.asarray(m, np.float64).ravel() for m in motion]))
            self._L.orc_add_triangles_moving(self._h, _dp(v), _dp(n), len(v), _dp(c9))

    def step(self):
        self._L.orc_step(self._h, 1)

    def steps(self, k):
        self._L.orc_step(self._h, int(k))

    def set_particle_material(self, youngs_modulus, poissons_ratio, density, friction_coefficient,
                              restitution_coefficient, surface_energy=0.0):
        self._L.orc_set_material(self._h, 0, youngs_modulus, poissons_ratio, density, friction_coefficient,
                                 restitution_coefficient, surface_energy)

    def set_wall_material(self, youngs_modulus, poissons_ratio, density, friction_coefficient,
                          restitution_coefficient, surface_energy=0.0):
        self._L.orc_set_material(self._h, 1, youngs_modulus, poissons_ratio, density, friction_coefficient,
                                 restitution_coefficient, surface_energy)

    def set_periodic_boundary(self, x, y, z):
        self._L.orc_set_periodic(self._h, int(bool(x)), int(bool(y)), int(bool(z)))

    def set_contact_models(self, normal, tangential):
        nm = NORMAL_MODELS.get(normal.lower())
        if nm is None:
            raise ValueError("Invalid normal force model")
        tm = TANGENTIAL_MODELS.get(tangential.lower())
        if tm is None:
            raise ValueError("Invalid tangential force model")
        self._L.orc_set_models(self._h, nm, tm)

    def run(self, duration):
        # steps = ceil(duration / dt) evaluated in f32 (src/lib.rs:356)
        n = int(math.ceil(float(np.float32(duration) / np.float32(self.dt))))
        self._L.orc_step(self._h, n)

    def get_particle_count(self):
        return int(self._L.orc_count(self._h))

    def _vec(self, which):
        n = self.get_particle_count()
        out = np.zeros((n, 3), np.float64)
        if n:
            self._L.orc_get_vec(self._h, which, _dp(out))
        return out

    def _set_vec(self, which, arr):
        arr = np.ascontiguousarray(arr, np.float64).reshape(-1, 3)
        self._L.orc_set_vec(self._h, which, _dp(arr))

    def _check(self, i):
        if i < 0 or i >= self.get_particle_count():
            raise IndexError("Particle index out of bounds")

    def get_particle_position(self, i):
        self._check(i)
        return tuple(self._vec(0)[i])

    def get_particle_velocity(self, i):
        self._check(i)
        return tuple(self._vec(1)[i])

    def get_particle_angular_velocity(self, i):
        self._check(i)
        return tuple(self._vec(3)[i])

    def set_particle_velocity(self, i, vx, vy, vz):
        self._check(i)
        v = self._vec(1)
        v[i] = (vx, vy, vz)
        self._set_vec(1, v)

    def set_particle_angular_velocity(self, i, x, y, z):
        self._check(i)
        w = self._vec(3)
        w[i] = (x, y, z)
        self._set_vec(3, w)

    # --- oracle extensions (diagnostics and state transfer) -------------
    def set_mode(self, mode):
        self._L.orc_set_mode(self._h, int(mode))

    def set_cell_size(self, h):
        self._L.orc_set_cell_size(self._h, float(h))

    def set_options(self, record_pairs=False, keep_contact_map=True, warn_stderr=False):
        self._L.orc_set_options(self._h, int(record_pairs), int(keep_contact_map), int(warn_stderr))

    def state(self):
        names = ["x", "v", "a", "w", "tau", "xres", "vres", "wres"]
        st = {k: self._vec(i) for i, k in enumerate(names)}
        n = self.get_particle_count()
        for i, k in enumerate(["r", "m", "fixed", "tag"]):
            out = np.zeros(n, np.float64)
            if n:
                self._L.orc_get_scalar(self._h, i, _dp(out))
            st[k] = out
        return st

    def set_state(self, st):
        for i, k in enumerate(["x", "v", "a", "w", "tau", "xres", "vres", "wres"]):
            if k in st:
                self._set_vec(i, st[k])

    def last_forces(self):
        n = self.get_particle_count()
        F = np.zeros((n, 3))
        T = np.zeros((n, 3))
        if n:
            self._L.orc_last_forces(self._h, _dp(F), _dp(T))
        return F, T

    def last_force_scale(self):
        """Per-particle sums of |f_ij| and |r x f_ij| of the last step."""
        n = self.get_particle_count()
        FS = np.zeros(n)
        TS = np.zeros(n)
        if n:
            self._L.orc_last_force_scale(self._h, _dp(FS), _dp(TS))
        return FS, TS

    def grid(self, now=True):
        """Reference grid for the current positions: (dims, cell per particle, flattened order)."""
        if now and self._L.orc_grid_now(self._h) != 0:
            raise RuntimeError("grid too large")
        d = (ctypes.c_int * 3)()
        self._L.orc_grid_dims(self._h, d)
        n = self.get_particle_count()
        cell = np.zeros(max(n, 1), np.int64)
        order = np.zeros(max(n, 1), np.int64)
        k = self._L.orc_grid_items(self._h, _lp(cell), _lp(order))
        return tuple(d), cell[:n], order[:k]

    def pairs(self):
        k = self._L.orc_pair_count(self._h)
        pi = np.zeros(max(k, 1), np.int64)
        pj = np.zeros(max(k, 1), np.int64)
        if k:
            self._L.orc_pairs(self._h, _lp(pi), _lp(pj))
        return pi[:k], pj[:k]

    def overlap_warnings(self):
        return int(self._L.orc_overlap_warnings(self._h))

    def contact_map_size(self):
        return int(self._L.orc_contact_map_size(self._h))


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def triangle_query(v9, n3, c, r, prec=64):
    v9 = np.ascontiguousarray(v9, np.float64)
    n3 = np.ascontiguousarray(n3, np.float64)
    c = np.ascontiguousarray(c, np.float64)
    pen = ctypes.c_double()
    nrm = np.zeros(3)
    hit = lib().orc_triangle_query(prec, _dp(v9), _dp(n3), _dp(c), float(r), ctypes.byref(pen), _dp(nrm))
    return (pen.value, nrm) if hit else None


def jkr_force(overlap, es, rs, gamma):
    """Normal force magnitude of the reference's JKR law in FP64 (src/physics.rs:132-219)."""
    return float(lib().orc_jkr_force(float(overlap), float(es), float(rs), float(gamma)))


def jkr_radius(overlap, es, rs, gamma):
    """(a, loop bodies run) of the reference's Newton iteration in FP64 (src/physics.rs:164-191)."""
    it = ctypes.c_int()
    a = lib().orc_jkr_radius(float(overlap), float(es), float(rs), float(gamma), ctypes.byref(it))
    return float(a), int(it.value)
