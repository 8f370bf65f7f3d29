"""Learned JKR contact radius on the GPU.

* The training samples' labels are the reference's own Newton iteration
  (src/physics.rs:164-191) bit for bit (oracle on the same FP64 inputs).
* The hand-written forward/backward kernels give the gradient of the numpy
  oracle (FP64) to FP32 accuracy; the tensor-core inference matches the
  quantised numpy forward pass.
* Trained on the GPU, the network drives the step: forces agree with the FP64
  oracle to 1e-6 of the term magnitudes (the target is 1e-5), and the test
  records what the network gains over the same certified solver without it
  (FP32 Newton steps per contact) and over the reference's Newton (force time).
"""
import ctypes

import numpy as np
import pytest

import parity_util as pu
from oracle import jkr_mlp as M

pytestmark = pytest.mark.gpu

# the adhesive workload's material: E = 5e8 Pa, nu = 0.25, rho = 2000,
# friction 0.5, restitution 0.5, surface energy 0.05 J/m^2
MAT = (5e8, 0.25, 2000.0, 0.5, 0.5, 0.05)


@pytest.fixture(scope="module")
def rp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rusty_particles_gb300 as m
    return m


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def test_samples_are_reference_newton_bit_exact(rp, oracle_mod):
    from oracle import oracle as O
    L = rp._lib.load()
    dom = np.array([2.5e-6, 1e-5, 2.0e8, 3.4e8, 0.04, 0.06, -0.1, 0.2])
    n = 4096
    feat = np.zeros((n, 4), np.float32)
    t = np.zeros(n, np.float32)
    w = np.zeros(n, np.float32)
    a = np.zeros(n)
    it = np.zeros(n, np.int32)
    inp = np.zeros((n, 4))
    rp._lib.check(L.rp_jkr_samples(_dp(dom), 7, n, _fp(feat), _fp(t), _fp(w), _dp(a),
                                   it.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dp(inp)))
    nconv = 0
    mismatch = 0
    for i in range(n):
        ov, rs, es, gamma = inp[i]
        ao, io = O.jkr_radius(ov, es, rs, gamma)
        assert a[i] == ao, (i, a[i], ao)
        assert abs(it[i]) % 100 == io or it[i] == io
        x, c = M.dims(ov, es, rs, gamma)
        cls = M.certify(x, c, ov > 0)
        if w[i] > 0:
            nconv += 1
            assert it[i] == io < 20
            # the reference's iterate is the root of the contact-radius relation
            u = M.root(x, c)
            assert abs(ao / rs - u) <= 1e-6 * u
            tt = M.target(ao, rs, x, c)
            assert abs(t[i] - tt) <= 1e-5 * (1 + abs(tt))
            f = M.features(x, c, rs, es, gamma)
            assert np.allclose(feat[i], f, rtol=1e-5, atol=1e-5)
        # FP32 certificate on the device vs real-arithmetic one: they can only
        # differ on the thresholds themselves
        mismatch += int((w[i] > 0) != (cls == 2))
    assert nconv > n // 2
    assert mismatch <= n // 500


def _net_inputs(seed, n):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.25, M.NPARAM).astype(np.float32)
    X = rng.normal(0, 1, (n, 4)).astype(np.float32)
    T = rng.normal(0, 0.5, n).astype(np.float32)
    W = (rng.random(n) > 0.25).astype(np.float32)
    return p, X, T, W


@pytest.mark.parametrize("n", [64, 1024])
def test_gradient_matches_cpu_oracle(rp, n):
    L = rp._lib.load()
    p, X, T, W = _net_inputs(5, n)
    g = np.zeros(M.NPARAM, np.float32)
    loss = ctypes.c_double()
    rp._lib.check(L.rp_mlp_loss_grad(_fp(p), _fp(X), _fp(T), _fp(W), n, 0, _fp(g), ctypes.byref(loss)))
    lo, go = M.loss_grad(p.astype(np.float64), X.astype(np.float64), T.astype(np.float64), W.astype(np.float64))
    assert abs(loss.value - lo) <= 1e-5 * lo
    # per layer, relative to the layer's gradient norm (FP32 sums over n samples)
    for a, b in ((M.O_W1, M.O_B1), (M.O_B1, M.O_W2), (M.O_W2, M.O_B2), (M.O_B2, M.O_W3), (M.O_W3, M.O_B3),
                 (M.O_B3, M.O_W4), (M.O_W4, M.O_B4), (M.O_B4, M.NPARAM)):
        err = np.linalg.norm(g[a:b] - go[a:b]) / max(np.linalg.norm(go[a:b]), 1e-30)
        assert err <= 2e-5, (a, b, err)


def test_quantised_gradient_matches_cpu_oracle(rp):
    # qat: BF16 weights and layer inputs in the forward pass, straight-through
    # gradients; the device's tanh.approx can move an activation across a BF16
    # rounding boundary, so the agreement is looser
    L = rp._lib.load()
    p, X, T, W = _net_inputs(6, 512)
    g = np.zeros(M.NPARAM, np.float32)
    loss = ctypes.c_double()
    rp._lib.check(L.rp_mlp_loss_grad(_fp(p), _fp(X), _fp(T), _fp(W), 512, 1, _fp(g), ctypes.byref(loss)))
    lo, go = M.loss_grad(p.astype(np.float64), X.astype(np.float64), T.astype(np.float64), W.astype(np.float64),
                         qat=True)
    assert abs(loss.value - lo) <= 2e-2 * lo
    assert np.linalg.norm(g - go) <= 3e-2 * np.linalg.norm(go)


def test_tensor_core_inference_matches_quantised_forward(rp):
    L = rp._lib.load()
    p, X, _, _ = _net_inputs(8, 1000)  # 1000 rows: a ragged last warp
    y = np.zeros(1000, np.float32)
    rp._lib.check(L.rp_mlp_infer(_fp(p), _fp(X), 1000, _fp(y)))
    yo, _ = M.forward(p.astype(np.float64), X.astype(np.float64), qat=True)
    scale = 1.0 + np.abs(yo)
    assert np.max(np.abs(y - yo) / scale) <= 3e-2
    assert np.mean(np.abs(y - yo) / scale) <= 3e-3


def _jkr_bed(seed, n, side):
    # lattice spacing 20 um, radii 9.8-10.2 um: overlap/R* within about
    # +-0.17, the training range being [-0.1, 0.2] (pairs below -0.1 are
    # certified zero and need no network)
    lo, hi = (0.0, 0.0, 0.0), (side, side, side)
    st = pu.random_bed(seed, n, lo, hi, 9.8e-6, 10.2e-6, vscale=0.02, wscale=100.0, ascale=0.0, tscale=0.0,
                       jitter=0.03)
    st["mass"] = 2000.0 * 4.0 / 3.0 * np.pi * st["radius"] ** 3
    return st, lo, hi


@pytest.fixture(scope="module")
def trained(rp):
    """One network trained on the GPU for the 9.5-10.5 um bed."""
    st, lo, hi = _jkr_bed(70, 512, 2.0e-4)
    g = pu.gpu_sim(rp, st, 1e-9, lo, hi, 3, 0, material=MAT)
    rep = g.train_jkr_network(samples=1 << 18, epochs=16, seed=3)
    return g.get_jkr_network(), rep


def test_training_reaches_accuracy(trained):
    (_, norm, dom), rep = trained
    assert rep["valid_samples"] > rep["samples"] // 2
    # held-out error of the BF16 network in t = ln(a/R*) - ln sqrt(max(x,0)+c^(2/3));
    # two Newton steps take 1e-2 to ~1e-8
    assert rep["val_rms"] < 5e-3, rep
    assert rep["val_max"] < 0.1, rep
    assert np.all(dom[:4] <= dom[4:])


def _forces_vs_oracle(rp, oracle_mod, net, solver, precision=0, seed=71, periodic=(True, True, True)):
    params, norm, dom = net
    st, lo, hi = _jkr_bed(seed, 3000, 3.0e-4)
    o = pu.oracle_sim(oracle_mod, st, 1e-9, lo, hi, 3, 0, periodic=periodic, material=MAT)
    g = pu.gpu_sim(rp, st, 1e-9, lo, hi, 3, 0, periodic=periodic, material=MAT, precision=precision)
    g.set_jkr_network(params, norm, dom)
    g.set_jkr_solver(solver)
    o.step()
    g.step()
    so, sg = o.state(), g.get_state()
    np.testing.assert_array_equal(sg["position"], so["x"])
    Fo, To = o.last_forces()
    Fg, Tg = g.debug_forces()
    FS, TS = o.last_force_scale()
    m = FS > 0
    ef = np.linalg.norm(Fg - Fo, axis=1)[m] / FS[m]
    et = np.linalg.norm(Tg - To, axis=1)[m] / TS[m]
    return float(ef.max(initial=0)), float(et.max(initial=0)), g.jkr_counters()


@pytest.mark.parametrize("solver", ["learned", "certified"])
def test_learned_forces_match_fp64_oracle(rp, oracle_mod, trained, solver):
    ef, et, cnt = _forces_vs_oracle(rp, oracle_mod, trained[0], solver)
    # the reference's own iterate is within 4e-8 of the root; 1e-6 leaves room
    assert ef <= 1e-6 and et <= 1e-6, (ef, et, cnt)
    assert cnt["accepted"] > 1000 and cnt["zero"] > 1000, cnt
    assert cnt["fallback"] <= 0.05 * (cnt["accepted"] + cnt["zero"] + cnt["fallback"]), cnt
    if solver == "learned":
        assert cnt["network_rows"] >= cnt["accepted"] * 0.95, cnt
        # two polish steps per network prediction (rejected ones fall back)
        assert 2 * cnt["accepted"] <= cnt["fp32_newton_steps"] <= 2 * (cnt["accepted"] + cnt["fallback"]), cnt


@pytest.mark.parametrize("normal,solver", [(3, "certified"), (3, "learned"), (4, "newton")])
def test_dropped_zero_pairs_match_oracle(rp, oracle_mod, trained, normal, solver):
    # without debug recording, pairs certified to add exactly +-0 (JKR beyond
    # pull-off; sJKR below delta_c) are dropped in the filter: the step must
    # still match the oracle (velocities carry the forces of the step)
    params, norm, dom = trained[0]
    st, lo, hi = _jkr_bed(73, 3000, 3.0e-4)
    per = (True, True, True)
    o = pu.oracle_sim(oracle_mod, st, 1e-9, lo, hi, normal, 0, periodic=per, material=MAT)
    g = pu.gpu_sim(rp, st, 1e-9, lo, hi, normal, 0, periodic=per, material=MAT)
    g.set_debug(False)
    g.set_jkr_network(params, norm, dom)
    g.set_jkr_solver(solver)
    o.steps(2)
    g.steps(2)
    so, sg = o.state(), g.get_state()
    FS, TS = o.last_force_scale()
    np.testing.assert_array_equal(np.isfinite(sg["velocity"]), np.isfinite(so["v"]))
    # forces within 1e-6 of each particle's sum of contact-force magnitudes,
    # over two steps of dt
    dt = 1e-9
    inertia = 0.4 * st["mass"] * st["radius"] ** 2
    tv = 4e-6 * FS / st["mass"] * dt + 1e-15
    tw = 4e-6 * TS / inertia * dt + 1e-12
    assert np.all(np.abs(sg["velocity"] - so["v"]).max(1) <= tv)
    assert np.all(np.abs(sg["angular_velocity"] - so["w"]).max(1) <= tw)
    assert np.all(np.abs(sg["position"] - so["x"]).max(1) <= tv * dt + 1e-18)


def test_learned_mixed_precision_within_1e5(rp, oracle_mod, trained):
    ef, et, cnt = _forces_vs_oracle(rp, oracle_mod, trained[0], "learned", precision=1)
    assert ef <= 1e-5 and et <= 1e-5, (ef, et, cnt)


def test_network_gain_over_method_without_it(rp, trained):
    """What the trained network buys: the certified solver without it needs
    the FP32 Newton iteration from the reference's start; with it, two steps
    from the prediction reach the same FP64-accepted root. Also times the
    force pass of the three solvers on one state."""
    params, norm, dom = trained[0]
    st, lo, hi = _jkr_bed(72, 20000, 5.4e-4)
    res = {}
    for solver in ("newton", "certified", "learned"):
        g = pu.gpu_sim(rp, st, 1e-9, lo, hi, 3, 0, periodic=(True, True, True), material=MAT)
        g.set_debug(False)
        g.set_jkr_network(params, norm, dom)
        g.set_jkr_solver(solver)
        g._L.rp_set_profiling(g._h, 1)
        g.steps(3)
        s0 = g.stats()
        g.steps(20)
        s1 = g.stats()
        c = g.jkr_counters()
        res[solver] = ((s1["force_ms"] - s0["force_ms"]) / max(s1["force_launches"] - s0["force_launches"], 1), c)
    cc, cl = res["certified"][1], res["learned"][1]
    steps_without = cc["fp32_newton_steps"] / max(cc["accepted"], 1)
    steps_with = cl["fp32_newton_steps"] / max(cl["accepted"], 1)
    print(f"\nFP32 Newton steps per converging contact: without network {steps_without:.2f}, "
          f"with network {steps_with:.2f}")
    print("force pass ms: " + ", ".join(f"{k} {v[0]:.4f}" for k, v in res.items()))
    assert abs(steps_with - 2.0) < 0.01
    assert steps_without >= 1.5 * steps_with, (steps_without, steps_with)
    # certificates and the FP32 solve remove the reference's FP64 iterations;
    # the network itself costs more than the FP32 Newton steps it saves on this
    # GPU (its pass is tens of microseconds, the saved steps about one), so
    # learned is not asserted to beat certified: the finding is reported
    assert res["learned"][0] < res["newton"][0], res
    assert res["certified"][0] < res["newton"][0], res
    print(f"learned / certified force pass: {res['learned'][0] / res['certified'][0]:.3f}")
