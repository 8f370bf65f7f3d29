"""Binary/ASCII STL writers used by the tests (format as written by
pydem/test_analytical_rotation.py:55-84: 80-byte header, u32 count,
50-byte records of normal + 3 vertices as little-endian f32 + u16)."""
import struct

import numpy as np


def write_binary_stl(path, tris):
    """tris: iterable of (v1, v2, v3); the normal is (v2-v1)x(v3-v1) normalised."""
    tris = [tuple(np.asarray(v, np.float64) for v in t) for t in tris]
    with open(path, "wb") as f:
        f.write(b"\x00" * 80)
        f.write(struct.pack("<I", len(tris)))
        for v1, v2, v3 in tris:
            n = np.cross(v2 - v1, v3 - v1)
            n = n / np.linalg.norm(n)
            f.write(struct.pack("<3f", *n))
            f.write(struct.pack("<3f", *v1))
            f.write(struct.pack("<3f", *v2))
            f.write(struct.pack("<3f", *v3))
            f.write(struct.pack("<H", 0))


def write_ascii_stl(path, tris, name="test"):
    with open(path, "w") as f:
        f.write(f"solid {name}\n")
        for v1, v2, v3 in tris:
            v1, v2, v3 = (np.asarray(v, np.float64) for v in (v1, v2, v3))
            n = np.cross(v2 - v1, v3 - v1)
            n = n / np.linalg.norm(n)
            f.write(f"  facet normal {n[0]:.9e} {n[1]:.9e} {n[2]:.9e}\n    outer loop\n")
            for v in (v1, v2, v3):
                f.write(f"      vertex {v[0]:.9e} {v[1]:.9e} {v[2]:.9e}\n")
            f.write("    endloop\n  endfacet\n")
        f.write(f"endsolid {name}\n")


def floor_tris():
    """The two floor triangles of pydem/test_analytical_rotation.py:184-200 (normal +Y)."""
    a = [(-10.0, 0.0, -10.0), (-10.0, 0.0, 10.0), (10.0, 0.0, -10.0)]
    b = [(10.0, 0.0, -10.0), (-10.0, 0.0, 10.0), (10.0, 0.0, 10.0)]
    return [a, b]


def box_tris(lo, hi):
    """12 inward-facing triangles of an axis-aligned box (reflecting walls)."""
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    c = [np.array([hi[0] if i & 1 else lo[0], hi[1] if i & 2 else lo[1], hi[2] if i & 4 else lo[2]]) for i in range(8)]
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    centre = (lo + hi) / 2
    out = []
    for q in quads:
        p = [c[k] for k in q]
        for t in ((p[0], p[1], p[2]), (p[0], p[2], p[3])):
            n = np.cross(t[1] - t[0], t[2] - t[0])
            if np.dot(n, centre - t[0]) < 0:
                t = (t[0], t[2], t[1])
            out.append(t)
    return out
