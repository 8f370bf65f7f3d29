"""numpy restatement of the wall contacts' triangle grid (test infrastructure).

The library builds the grid on the device (csrc/k_trigrid.cu with the set-up
in Engine::build_triangle_grid); this module builds the same grid with the
same double arithmetic (numpy fuses no multiply-adds), so the two can be
compared bit for bit: the grown boxes, the cell size chosen by the same
sequence of trials, the distance pruning of each (triangle, cell) candidate by
the closest-point regions of Ericson, Real-Time Collision Detection (2005),
5.1.5, and the lists in mesh order.
"""
import math

import numpy as np


def _dot(u, w):
    return u[:, 0] * w[:, 0] + u[:, 1] * w[:, 1] + u[:, 2] * w[:, 2]


def point_triangle_dist2(p, a, b, c):
    """Squared distance from each p to its triangle (a, b, c); arrays [M, 3]."""
    with np.errstate(all="ignore"):
        out = np.full(len(p), np.nan)
        done = np.zeros(len(p), bool)

        def put(m, val):
            out[m] = val[m]
            done[m] = True

        ab, ac, ap = b - a, c - a, p - a
        d1, d2 = _dot(ab, ap), _dot(ac, ap)
        put((d1 <= 0) & (d2 <= 0), _dot(ap, ap))
        bp = p - b
        d3, d4 = _dot(ab, bp), _dot(ac, bp)
        put(~done & (d3 >= 0) & (d4 <= d3), _dot(bp, bp))
        vc = d1 * d4 - d3 * d2
        m = ~done & (vc <= 0) & (d1 >= 0) & (d3 <= 0)
        v = d1 / (d1 - d3)
        q = a + v[:, None] * ab
        put(m, _dot(p - q, p - q))
        cp = p - c
        d5, d6 = _dot(ab, cp), _dot(ac, cp)
        put(~done & (d6 >= 0) & (d5 <= d6), _dot(cp, cp))
        vb = d5 * d2 - d1 * d6
        m = ~done & (vb <= 0) & (d2 >= 0) & (d6 <= 0)
        w = d2 / (d2 - d6)
        q = a + w[:, None] * ac
        put(m, _dot(p - q, p - q))
        va = d3 * d6 - d5 * d4
        m = ~done & (va <= 0) & (d4 - d3 >= 0) & (d5 - d6 >= 0)
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6))
        q = b + w[:, None] * (c - b)
        put(m, _dot(p - q, p - q))
        den = 1.0 / (va + vb + vc)
        v, w = vb * den, vc * den
        q = a + ab * v[:, None] + ac * w[:, None]
        put(~done, _dot(p - q, p - q))
    return out


def triangle_grid(tri_v, rmax):
    """(dims, lo, cell, start, items) of the grid for float32 vertices [T, 9]."""
    v = np.asarray(tri_v, np.float32).astype(np.float64).reshape(-1, 3, 3)
    T = len(v)
    extent_abs = float(np.abs(v).max())
    grow = rmax * (1.0 + 1e-6) + 1e-6 * (1.0 + extent_abs + rmax)
    blo = v.min(1) - grow
    bhi = v.max(1) + grow
    lo, hi = blo.min(0), bhi.max(0)
    ext = float((hi - lo).max())
    cell = max(rmax, ext / 1024.0)
    for _ in range(80):
        dims = np.maximum(1, np.ceil((hi - lo) / cell)).astype(np.int64)
        if int(np.prod(dims)) > (1 << 24):
            cell *= 1.5
            continue
        a = np.maximum(0, np.floor((blo - lo) / cell)).astype(np.int64)
        b = np.minimum(dims - 1, np.floor((bhi - lo) / cell)).astype(np.int64)
        if int(np.prod(b - a + 1, axis=1).sum()) <= 64 * T + (1 << 22):
            break
        cell *= 1.5
    a = np.maximum(0, np.floor((blo - lo) / cell)).astype(np.int64)
    b = np.minimum(dims - 1, np.floor((bhi - lo) / cell)).astype(np.int64)
    reach = cell * math.sqrt(3.0) * 0.5 + grow
    reach2 = reach * reach * (1.0 + 1e-9) + 1e-24
    n = b - a + 1
    counts = np.prod(n, axis=1)
    tri = np.repeat(np.arange(T), counts)
    local = np.arange(int(counts.sum())) - np.repeat(np.cumsum(counts) - counts, counts)
    nx, ny = n[tri, 0], n[tri, 1]
    x = a[tri, 0] + local % nx
    y = a[tri, 1] + (local // nx) % ny
    z = a[tri, 2] + local // (nx * ny)
    cc = np.stack([lo[0] + (x + 0.5) * cell, lo[1] + (y + 0.5) * cell, lo[2] + (z + 0.5) * cell], 1)
    e0, e1 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    cr = np.stack([e0[:, 1] * e1[:, 2] - e0[:, 2] * e1[:, 1], e0[:, 2] * e1[:, 0] - e0[:, 0] * e1[:, 2],
                   e0[:, 0] * e1[:, 1] - e0[:, 1] * e1[:, 0]], 1)
    ln = np.sqrt(_dot(cr, cr))
    flat = ~((ln > 0) & np.isfinite(ln))
    d2 = point_triangle_dist2(cc, v[tri, 0], v[tri, 1], v[tri, 2])
    keep = flat[tri] | ~(d2 > reach2)
    cellid = x + dims[0] * (y + dims[1] * z)
    ck, tk = cellid[keep], tri[keep]
    order = np.lexsort((tk, ck))  # by cell, triangles in mesh order
    ncells = int(np.prod(dims))
    start = np.zeros(ncells + 1, np.int64)
    np.add.at(start, ck + 1, 1)
    return tuple(int(d) for d in dims), lo, cell, np.cumsum(start), tk[order]
