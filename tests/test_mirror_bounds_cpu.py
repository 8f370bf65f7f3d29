"""The inner intervals of the integrator's wrap and removal tests (built in
Engine::build_params, read by k_first_half in rusty_particles_gb300/csrc/k_step.cu),
restated in numpy: when the FP32 mirror of a position lies strictly inside an
axis's inner interval, the FP64 position needs no periodic wrap (it is inside
[bmin, bmax)) or is kept (it is inside [bmin - 1, bmax + 1] on an open axis), so
skipping the FP64 comparisons changes no decision. Checked on random boxes with
positions packed around every face, at the last floats inside the intervals.
(Rounding to FP32 is monotone, so a mirror above the rounded bound already puts
the FP64 position above the bound; the margin of 1e-6 (|bounds| + 2) is spare.
An interval one float wider than the rounded bound fails this test.)
"""
import numpy as np


def inner_intervals(bmin, bmax, periodic):
    bmag = max(max(abs(a), abs(b)) for a, b in zip(bmin, bmax))
    m = 1e-6 * (bmag + 2.0)
    lo, hi = [], []
    for k in range(3):
        l_ = bmin[k] + m if periodic[k] else bmin[k] - 1.0 + m
        h_ = bmax[k] - m if periodic[k] else (np.inf if k == 1 else bmax[k] + 1.0 - m)
        lo.append(np.nextafter(np.float32(l_), np.float32(np.inf)))
        hi.append(np.float32(np.inf) if np.isinf(h_) else np.nextafter(np.float32(h_), np.float32(-np.inf)))
    return lo, hi


def test_inside_the_inner_interval_decides_like_fp64():
    rng = np.random.default_rng(8)
    for trial in range(200):
        scale = 10.0 ** rng.uniform(-2, 3)
        bmin = rng.uniform(-2, 0, 3) * scale
        bmax = bmin + rng.uniform(0.01, 2, 3) * scale
        periodic = rng.integers(0, 2, 3).astype(bool)
        lo, hi = inner_intervals(bmin, bmax, periodic)
        for k in range(3):
            faces = [bmin[k], bmax[k]] if periodic[k] else [bmin[k] - 1.0, bmax[k] + 1.0]
            x = np.concatenate([f + rng.normal(0, 1, 20000) * 10.0 ** rng.uniform(-12, -2) * max(1.0, abs(f))
                                for f in faces])
            edges = [np.float64(lo[k])] + ([np.float64(hi[k])] if np.isfinite(hi[k]) else [])
            x = np.concatenate([x, np.array(edges)])
            xf = x.astype(np.float32)
            inside = (xf > lo[k]) & (xf < hi[k])
            if periodic[k]:
                ok = (x >= bmin[k]) & (x < bmax[k])
            elif k == 1:
                ok = x >= bmin[k] - 1.0
            else:
                ok = (x >= bmin[k] - 1.0) & (x <= bmax[k] + 1.0)
            assert np.all(ok[inside]), (trial, k)
