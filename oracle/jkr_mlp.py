"""CPU oracle of the learned JKR contact radius (test infrastructure only).

Two parts, both in float64 numpy:

* The 4-64-64-64-1 tanh network the GPU trains: forward pass, mean-squared
  loss and its analytic gradient, with an optional emulation of the inference
  arithmetic (BF16 weights and layer inputs, round to nearest even) and
  straight-through gradients. The GPU's forward/backward kernels are checked
  against ``loss_grad``; ``loss_grad`` itself is checked against central
  finite differences.
* The exact certificates on the reference's JKR Newton iteration
  (src/physics.rs:164-191) in real arithmetic, and the features / target of
  the network, so tests can confirm that the iteration really converges where
  the certificate says it does and returns zero where it says so.

Parameter layout (float32 on the device): W1[64][4] b1[64] W2[64][64] b2[64]
W3[64][64] b3[64] W4[64] b4, rows = outputs.
"""
from __future__ import annotations

import numpy as np

H = 64
NPARAM = H * 4 + H + 2 * (H * H + H) + H + 1  # 8705
O_W1, O_B1 = 0, 256
O_W2, O_B2 = 320, 4416
O_W3, O_B3 = 4480, 8576
O_W4, O_B4 = 8640, 8704

KAPPA = 16.0 ** (-1.0 / 6.0) - 16.0 ** (-2.0 / 3.0)  # min of u^2 - sqrt(c u) is -KAPPA c^(2/3)
XI_NEG, XI_POS, XI_WALK = -0.4525, 0.16, 0.155
C_MIN, C_MAX = 1e-6, 0.1


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    out = (r << 16).astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out = np.where(nan, np.nan, out)
    return out


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[O_W1:O_B1].reshape(H, 4), p[O_B1:O_W2], p[O_W2:O_B2].reshape(H, H), p[O_B2:O_W3],
            p[O_W3:O_B3].reshape(H, H), p[O_B3:O_W4], p[O_W4:O_B4], p[O_B4])


def forward(p, X, qat=False):
    """Network output for rows X (n x 4); returns (y, cache)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p)
    q = bf16 if qat else (lambda a: np.asarray(a, np.float64))
    if qat:
        W1, W2, W3, W4 = q(W1), q(W2), q(W3), q(W4)
    x0 = q(X)
    h1 = np.tanh(x0 @ W1.T + b1)
    h2 = np.tanh(q(h1) @ W2.T + b2)
    h3 = np.tanh(q(h2) @ W3.T + b3)
    y = q(h3) @ W4 + b4
    return y, (x0, h1, h2, h3, W2, W3, W4, q)


def loss_grad(p, X, T, Wt, qat=False):
    """sum_s w_s (y_s - t_s)^2 / n and its gradient (straight-through under qat)."""
    n = X.shape[0]
    y, (x0, h1, h2, h3, W2, W3, W4, q) = forward(p, X, qat)
    e = y - T
    loss = float(np.sum(Wt * e * e) / n)
    dy = 2.0 * Wt * e / n
    g = np.zeros(NPARAM)
    g[O_W4:O_B4] = dy @ q(h3)
    g[O_B4] = dy.sum()
    d3 = np.outer(dy, W4) * (1.0 - h3 * h3)
    g[O_W3:O_B3] = (d3.T @ q(h2)).ravel()
    g[O_B3:O_W4] = d3.sum(0)
    d2 = (d3 @ W3) * (1.0 - h2 * h2)
    g[O_W2:O_B2] = (d2.T @ q(h1)).ravel()
    g[O_B2:O_W3] = d2.sum(0)
    d1 = (d2 @ W2) * (1.0 - h1 * h1)
    g[O_W1:O_B1] = (d1.T @ x0).ravel()
    g[O_B1:O_W2] = d1.sum(0)
    return loss, g


def finite_difference(p, X, T, Wt, idx, h=1e-6):
    """Central differences of loss_grad's loss (qat off) at parameter indices idx."""
    p = np.asarray(p, np.float64).copy()
    out = np.zeros(len(idx))
    for k, i in enumerate(idx):
        old = p[i]
        p[i] = old + h
        lp, _ = loss_grad(p, X, T, Wt)
        p[i] = old - h
        lm, _ = loss_grad(p, X, T, Wt)
        p[i] = old
        out[k] = (lp - lm) / (2 * h)
    return out


# ------------------------------------------------------------- certificates
def dims(overlap, es, rs, gamma):
    """x = overlap/R*, c = C/R* with C = 8 pi gamma / E* (the reference's c_val)."""
    C = 8.0 * np.pi * gamma / es
    return overlap / rs, C / rs


def certify(x, c, pos):
    """0 = the reference's Newton must run, 1 = it returns zero force, 2 = it
    converges to the root on the increasing branch, 3 = it only halves its
    start sqrt(x) (the clamp binds at every step) (real arithmetic; the
    device adds FP32 rounding margins)."""
    c23 = c ** (2.0 / 3.0)
    if x + KAPPA * c23 + 1e-3 < -1e-5 * (abs(x) + c23 + 1e-3):
        return 1
    if not (C_MIN <= c <= C_MAX):
        return 0
    xi = x / c23
    if pos:
        return 2 if xi >= XI_POS else (3 if xi <= XI_WALK else 0)
    return 2 if xi >= XI_NEG else 0


def walk_radius(overlap, rs):
    """Where the reference's loop ends in the halving region: sqrt(R* delta)
    halved until the step falls below 1e-6 R* (at most 20 times)."""
    a = np.sqrt(rs * overlap)
    lim = 1e-6 * rs
    for _ in range(20):
        st = a * 0.5
        a = a - st
        if st < lim:
            break
    return a


def features(x, c, rs, es, gamma):
    """sqrt(xi + kappa) with xi = x / c^(2/3), ln R*, ln E*, ln gamma."""
    c23 = c ** (2.0 / 3.0)
    return np.array([np.sqrt(max(x / c23 + KAPPA, 0.0)), np.log(rs), np.log(es), np.log(gamma)])


def target(a, rs, x, c):
    """t = ln(a/R*) - ln sqrt(max(x,0) + c^(2/3))."""
    return np.log(a / rs) - 0.5 * np.log(max(x, 0.0) + c ** (2.0 / 3.0))


def root(x, c):
    """The larger root u of u^2 - sqrt(c u) = x by bisection (float64)."""
    lo = (c / 16.0) ** (1.0 / 3.0)  # minimum of the left side
    hi = max(1.0, 2.0 * np.sqrt(abs(x) + 1.0))
    for _ in range(200):
        m = 0.5 * (lo + hi)
        if m * m - np.sqrt(c * m) - x > 0:
            hi = m
        else:
            lo = m
    return 0.5 * (lo + hi)
