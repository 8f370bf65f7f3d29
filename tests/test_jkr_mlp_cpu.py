"""CPU checks of the learned-JKR oracle: the numpy network gradient against
finite differences, BF16 rounding, and the two certificates on the
reference's Newton iteration (src/physics.rs:164-191) run by the C oracle."""
import numpy as np
import pytest

from oracle import jkr_mlp as M


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, M.NPARAM)
    X = rng.normal(0, 1, (64, 4))
    T = rng.normal(0, 1, 64)
    W = (rng.random(64) > 0.2).astype(float)
    _, g = M.loss_grad(p, X, T, W)
    idx = np.concatenate([rng.choice(M.NPARAM, 80, replace=False), [M.O_W1, M.O_B1 + 3, M.O_W4 + 7, M.O_B4]])
    fd = M.finite_difference(p, X, T, W, idx)
    assert np.max(np.abs(fd - g[idx])) <= 1e-7 * np.max(np.abs(g[idx]))


def test_bf16_rounding_nearest_even():
    # 1 + 2^-8 is halfway between two BF16 values: ties go to the even one (1.0)
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e38, 1e-40], np.float32)
    out = M.bf16(vals)
    assert out[0] == 1.0 and out[1] == 1.0 and out[2] == 1.0 + 2.0 ** -6
    assert out[3] == -2.5
    assert np.isfinite(out[4]) or out[4] == np.inf
    # subnormals keep the BF16 spacing 2^-133
    assert abs(out[5] - 1e-40) <= 0.5 * 2.0 ** -133


def test_qat_forward_equals_unquantised_on_bf16_grid():
    # with BF16-representable weights and inputs the quantised forward only
    # rounds the hidden activations
    rng = np.random.default_rng(3)
    p = M.bf16(rng.normal(0, 0.2, M.NPARAM).astype(np.float32))
    X = M.bf16(rng.normal(0, 1, (16, 4)).astype(np.float32))
    y0, _ = M.forward(p, X, qat=False)
    y1, _ = M.forward(p, X, qat=True)
    assert np.max(np.abs(y0 - y1)) < 0.05 * (1 + np.max(np.abs(y0)))


def _sweep(n, seed):
    rng = np.random.default_rng(seed)
    for trial in range(n):
        lc = rng.uniform(-6, -1)
        c = 10 ** lc
        rs = 10 ** rng.uniform(-7, -2)
        es = 10 ** rng.uniform(6, 11)
        gamma = c * rs * es / (8 * np.pi)
        if trial % 2:
            xi = rng.uniform(-0.7, 3.0)
        else:
            xi = 10 ** rng.uniform(-1, 4) * (1 if rng.random() < 0.75 else -1)
        yield xi * c ** (2.0 / 3.0) * rs, es, rs, gamma


def test_certificates_hold_for_reference_newton(oracle_mod):
    from oracle import oracle as O
    O.build()
    conv = zeros = 0
    worst_it = 0
    worst_rel = 0.0
    for ov, es, rs, gamma in _sweep(6000, 11):
        x, c = M.dims(ov, es, rs, gamma)
        cls = M.certify(x, c, ov > 0)
        a, it = O.jkr_radius(ov, es, rs, gamma)
        if cls == 2:
            conv += 1
            u = M.root(x, c)
            rel = abs(a / rs - u) / u
            worst_rel = max(worst_rel, rel)
            worst_it = max(worst_it, it)
            assert it < 20 and rel <= 1e-6, (ov, es, rs, gamma, it, rel)
        elif cls == 1:
            zeros += 1
            assert O.jkr_force(ov, es, rs, gamma) == 0.0, (ov, es, rs, gamma)
    assert conv > 3000 and zeros > 300
    # the reference's converged radius is within 4e-8 of the root (its last
    # step is < 1e-6 R*): the learned solver can agree with it to that level
    assert worst_rel < 1e-7 and worst_it <= 14


def test_halving_walk_is_closed_form(oracle_mod):
    # delta > 0 with the start left of the minimum: the reference's loop only
    # halves sqrt(R* delta); its end point is reproduced bit for bit
    from oracle import oracle as O
    O.build()
    rng = np.random.default_rng(5)
    n = 0
    for t in range(6000):
        c = 10 ** rng.uniform(-6, -1)
        rs = 10 ** rng.uniform(-7, -2)
        es = 10 ** rng.uniform(6, 11)
        gamma = c * rs * es / (8 * np.pi)
        xi = rng.uniform(1e-9, M.XI_WALK) if t % 3 else 10 ** rng.uniform(-12, np.log10(M.XI_WALK))
        ov = xi * c ** (2.0 / 3.0) * rs
        if not ov > 0:
            continue
        x, cc = M.dims(ov, es, rs, gamma)
        assert M.certify(x, cc, True) == 3
        a, _ = O.jkr_radius(ov, es, rs, gamma)
        assert M.walk_radius(ov, rs) == a
        n += 1
    assert n > 5000


def test_no_root_region_gives_zero_force_without_iterating(oracle_mod):
    from oracle import oracle as O
    O.build()
    es, gamma = 2.0e8, 0.05
    for rs in (2.5e-6, 1e-5, 1e-3):
        x, c = M.dims(0.0, es, rs, gamma)
        c23 = c ** (2.0 / 3.0)
        gmin = -M.KAPPA * c23
        for x in np.linspace(gmin - 1e-3 - 0.5, gmin - 1.001e-3, 50):
            assert M.certify(x, c, False) == 1
            assert O.jkr_force(x * rs, es, rs, gamma) == 0.0


@pytest.mark.parametrize("xi", [0.2, 1.0, 30.0, -0.3, -0.45])
def test_target_recovers_root(xi):
    c = 1e-3
    rs, es = 5e-6, 2.7e8
    gamma = c * rs * es / (8 * np.pi)
    x = xi * c ** (2.0 / 3.0)
    u = M.root(x, c)
    t = M.target(u * rs, rs, x, c)
    ub = np.sqrt(max(x, 0.0) + c ** (2.0 / 3.0))
    assert abs(np.exp(t) * ub - u) <= 1e-12 * u
    f = M.features(x, c, rs, es, gamma)
    assert abs(f[0] - np.sqrt(xi + M.KAPPA)) < 1e-12
