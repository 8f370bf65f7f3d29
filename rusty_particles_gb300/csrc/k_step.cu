// Per-step kernels of the DEM step: the first-half kernel (the previous
// step's second half kick, boundary rule, half kick + drift), the pair/wall
// force gather, the end-of-step bookkeeping and the closing second half kick.
//
// This translation unit is compiled with -fmad=false: every double operation
// rounds exactly as the oracle's (-ffp-contract=off), so positions after the
// first half, cutoff decisions, normals and relative velocities are
// bit-identical to the reference algorithm evaluated in FP64 from the same
// state. Force magnitudes differ only where a transcendental is evaluated
// differently (delta^1.5 as delta*sqrt(delta)), well inside 1e-9 relative.
//
// Precision forms of the pair force (StepParams::prec):
//   FP64  — all pair math in double.
//   MIXED — the cutoff decision, r_sum^2 - d^2 (the overlap without
//           cancellation) and v_i - v_j stay in double; normals, relative
//           velocity, force laws and torques run in float; the per-particle
//           force/torque sums, the state and the integrator stay in double.
#include <cfloat>

#include "rp_device.cuh"
#include "rp_launch.h"
#include "rp_mlp.cuh"

namespace rp {

template <typename R>
struct T3 {
  R x, y, z;
};
template <typename R> __device__ __forceinline__ T3<R> t3(R x, R y, R z) { return T3<R>{x, y, z}; }
template <typename R> __device__ __forceinline__ T3<R> operator+(T3<R> a, T3<R> b) { return T3<R>{a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R> __device__ __forceinline__ T3<R> operator-(T3<R> a, T3<R> b) { return T3<R>{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R> __device__ __forceinline__ T3<R> operator-(T3<R> a) { return T3<R>{-a.x, -a.y, -a.z}; }
template <typename R> __device__ __forceinline__ T3<R> operator*(T3<R> a, R s) { return T3<R>{a.x * s, a.y * s, a.z * s}; }
template <typename R> __device__ __forceinline__ T3<R> operator*(R s, T3<R> a) { return T3<R>{s * a.x, s * a.y, s * a.z}; }
template <typename R> __device__ __forceinline__ T3<R> operator/(T3<R> a, R s) { return T3<R>{a.x / s, a.y / s, a.z / s}; }
template <typename R> __device__ __forceinline__ R dot(T3<R> a, T3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> __device__ __forceinline__ T3<R> cross(T3<R> a, T3<R> r) {
  return T3<R>{a.y * r.z - r.y * a.z, a.z * r.x - r.z * a.x, a.x * r.y - r.x * a.y};
}
template <typename R> __device__ __forceinline__ R len(T3<R> a) { return sqrt(dot(a, a)); }
template <typename R, typename S> __device__ __forceinline__ T3<R> cvt(T3<S> a) { return T3<R>{(R)a.x, (R)a.y, (R)a.z}; }

using V = T3<double>;
using Vf = T3<float>;
__device__ __forceinline__ V vmk(double x, double y, double z) { return V{x, y, z}; }
__device__ __forceinline__ V xyz(const D4& d) { return V{d.x, d.y, d.z}; }
// isfinite(x) and 0.0 + x from the bits, off the FP64 pipe
__device__ __forceinline__ bool finite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000; }
__device__ __forceinline__ double plus_zero(double x) {
  return (__double_as_longlong(x) << 1) == 0 ? 0.0 : x;
}
__device__ __forceinline__ float plus_zero(float x) { return (__float_as_int(x) << 1) == 0 ? 0.0f : x; }

constexpr double kPi = 3.14159265358979323846;

// float -> double, exactly, on the integer pipe: a normal float's exponent is
// re-biased (+896) and its mantissa shifted into place; zeros keep their sign.
// Subnormals, infinities and NaNs take the hardware conversion, which runs on
// the FP64 pipe like every FP64 instruction.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  if ((u << 1) == 0u) return __longlong_as_double((long long)((uint64_t)u << 32));
  if (e == 0u || e == 0xFFu) return (double)f;
  return __longlong_as_double((long long)(((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                                          ((uint64_t)(u & 0x7FFFFFu) << 29)));
}

// ------------------------------------------------------------- force laws
// src/physics.rs:49-70
template <typename R>
__device__ __forceinline__ R lsd_mag(R overlap, R vn, R kn, R gn) {
  return fmax(kn * overlap - gn * vn, R(0));
}
// src/physics.rs:86-129. With s = sqrt(R* delta): the elastic term
// (4/3) E* sqrt(R*) delta^1.5 = (4/3) E* s delta and the tangent stiffness
// 2 E* sqrt(R* delta) = 2 E* s share one square root.
template <typename R>
__device__ __forceinline__ R hertz_mag(R overlap, R vn, R es, R rs, R ms, R beta_abs) {
  if (overlap <= R(0)) return R(0);
  R s = sqrt(rs * overlap);
  R fe = R(4.0 / 3.0) * es * s * overlap;
  R kt = R(2) * es * s;
  R cn = R(2) * sqrt(ms * kt) * beta_abs;
  R fd = -cn * vn;
  return fmax(fe + fd, R(0));
}
template <typename R>
__device__ __forceinline__ R hertz_elastic_mag(R overlap, R es, R rs) {
  R kn = R(4.0 / 3.0) * es * sqrt(rs);
  return overlap > R(0) ? kn * (overlap * sqrt(overlap)) : R(0);
}
// src/physics.rs:132-219 (Newton on a^2/R* - sqrt(C a) - delta = 0).
// `near` (FP32 callers) is set when a cut-off decision lies within rounding.
template <typename R>
__device__ __forceinline__ R jkr_mag(R overlap, R es, R rs, R gamma, bool* near = nullptr) {
  if (gamma <= R(0)) return hertz_elastic_mag(overlap, es, rs);
  const R eight_pi = R(8) * R(kPi);
  R c_val = eight_pi * gamma / es;
  R sqrt_c = sqrt(c_val);
  R a = overlap > R(0) ? sqrt(rs * overlap) : rs * R(0.5);
  for (int it = 0; it < 20; ++it) {
    if (a <= R(0)) a = R(1e-9);
    R ts = sqrt(c_val * a);
    R f_val = a * a / rs - ts - overlap;
    R df = R(2) * a / rs - R(0.5) * sqrt_c / sqrt(a);
    if (fabs(df) < R(1e-9)) break;
    R da = f_val / df;
    R max_step = a * R(0.5);
    R step = da;
    if (step < -max_step) step = -max_step;
    if (step > max_step) step = max_step;
    a = a - step;
    if (fabs(step) < R(1e-6) * rs) break;
  }
  R ts = sqrt(c_val * a);
  R f_val = a * a / rs - ts - overlap;
  if (near && fabs(fabs(f_val) - R(1e-3) * rs) <= R(1e-5) * rs) *near = true;
  if (fabs(f_val) > R(1e-3) * rs) return R(0);
  if (a <= R(0)) return R(0);
  R a3 = a * a * a;
  R term1 = R(4) * es * a3 / (R(3) * rs);
  R term2 = sqrt(eight_pi * gamma * es * a3);
  R fm = term1 - term2;
  R f_pull = R(-2.0 / 3.0) * R(kPi) * gamma * rs;
  if (near && fabs(fm - f_pull) <= R(1e-5) * (term1 + term2)) *near = true;
  if (fm < f_pull) return R(0);
  return fm;
}
// JKR magnitude of a particle pair without the reference's Newton loop, or
// JKR_FALLBACK when that loop must run (P.jkr_solver 1 or 2). The
// certificates (rp_mlp.cuh) either prove the reference returns zero or that
// its iteration converges to the root on the increasing branch; the root is
// then found in FP32 (solver 1: two Newton steps from the network's `guess`;
// solver 2: Newton from the reference's own start), accepted only when its
// FP64 residual is <= 1e-6 of the terms, corrected by one FP64-accurate Newton
// step, and turned into the reference's force 4 E* a^3/(3 R*) - sqrt(8 pi
// gamma E* a^3) = E* a (4 a^2/(3 R*) - sqrt(C a)). The pull-off cut is decided
// in FP64 and left to the reference's loop when within 1e-7 of the terms.
__device__ __forceinline__ int jkr_learned(const StepParams& P, const Law& L, double overlap, double rs, float guess,
                                           double& fm, uint32_t& iters) {
  const float rsf = (float)rs;
  const float x = (float)overlap / rsf;
  const float c = L.jkr_Cf / rsf;
  const float c23 = jkr_c23(c);
  const int cls = jkr_certify(x, c, c23, overlap > 0.0);
  if (cls == JKR_ZERO) {
    fm = 0.0;
    return JKR_ZERO;
  }
  if (cls == JKR_WALK) {
    // the reference's halving walk, then its own tail (src/physics.rs:193-218),
    // operation for operation in FP64
    const double es = L.es_pp, gamma = L.gamma_pp;
    const double eight_pi = 8.0 * kPi;
    const double c_val = eight_pi * gamma / es;
    double a = sqrt(rs * overlap);
    const double lim = 1e-6 * rs;
    for (int it = 0; it < 20; ++it) {
      const double st = a * 0.5;
      a = a - st;
      if (st < lim) break;
    }
    const double ts = sqrt(c_val * a);
    const double f_val = a * a / rs - ts - overlap;
    fm = 0.0;
    if (fabs(f_val) > 1e-3 * rs || a <= 0.0) return JKR_WALK;
    const double a3 = a * a * a;
    const double term1 = 4.0 * es * a3 / (3.0 * rs);
    const double term2 = sqrt(eight_pi * gamma * es * a3);
    const double fmv = term1 - term2;
    const double f_pull = (-2.0 / 3.0) * kPi * gamma * rs;
    fm = fmv < f_pull ? 0.0 : fmv;
    return JKR_WALK;
  }
  if (cls != JKR_CONVERGES) return JKR_FALLBACK;
  float u;
  if (P.jkr_solver == 1) {
    if (!(guess > 0.0f && guess < 1e30f)) return JKR_FALLBACK;
    u = jkr_newton_f32(jkr_newton_f32(guess, x, c), x, c);
    iters += 2;
  } else {
    u = overlap > 0.0 ? sqrtf(x) : 0.5f;
    for (int k = 0; k < 40; ++k) {
      const float un = jkr_newton_f32(u, x, c);
      ++iters;
      const bool done = fabsf(un - u) <= 1e-6f * un;
      u = un;
      if (done) break;
    }
  }
  // FP64 residual of a = u R*: sqrt(C a) from the FP32 root plus one Newton
  // step of the square root (error ~1e-14), no FP64 division
  const double ud = (double)u;
  const double Ca = L.jkr_C * (ud * rs);
  const float s0 = sqrtf((float)Ca);
  if (!(s0 > 0.0f)) return JKR_FALLBACK;
  const double ts = (double)s0 + (Ca - (double)s0 * (double)s0) * (double)(0.5f / s0);
  const double uu = ud * ud * rs;  // a^2 / R*
  const double f = uu - ts - overlap;
  if (!(fabs(f) <= 1e-6 * (uu + ts + fabs(overlap)))) return JKR_FALLBACK;
  const float dg = 2.0f * u - 0.5f * (float)ts / ((float)ud * rsf);
  if (!(dg > 0.0f)) return JKR_FALLBACK;
  const float du = (float)f / (rsf * dg);
  const double u1 = ud - (double)du;
  const float q = du / u;
  const double ts1 = ts * (1.0 - (double)(0.5f * q + 0.125f * q * q));
  const double es = L.es_pp;
  const double a1 = u1 * rs;
  const double term1 = (4.0 / 3.0) * es * (u1 * u1 * u1) * (rs * rs);
  const double term2 = es * a1 * ts1;
  const double fmv = term1 - term2;
  const double f_pull = (-2.0 / 3.0) * kPi * L.gamma_pp * rs;
  if (fabs(fmv - f_pull) <= 1e-7 * (term1 + term2)) return JKR_FALLBACK;
  fm = fmv < f_pull ? 0.0 : fmv;
  return JKR_CONVERGES;
}

// src/physics.rs:234-325
template <typename R>
__device__ __forceinline__ R sjkr_mag(R overlap, R vn, R es, R rs, R gamma) {
  if (gamma <= R(0)) return hertz_elastic_mag(overlap, es, rs);
  R f_pull = R(1.5) * R(kPi) * gamma * rs;
  R term = R(3) * (R(kPi) * R(kPi)) * (gamma * gamma) * rs / (es * es);
  R delta_c = -sqrt(term);
  if (overlap < delta_c) return R(0);
  R coh = vn > R(0) ? R(1) : R(0);
  R fh = overlap > R(0) ? R(4.0 / 3.0) * es * sqrt(rs) * (overlap * sqrt(overlap)) : R(0);
  return fh - coh * f_pull;
}

// Normal force vector for the configured model. The reference passes
// Vec3::ZERO as the relative velocity to the hysteretic particle-particle law
// (src/simulation.rs:409-411) and the real one for walls (:495-501).
template <typename R>
__device__ __forceinline__ R normal_mag(int model, R overlap, T3<R> n, T3<R> rv, R es, R rs, R ms, R beta_abs,
                                       R gamma, bool wall) {
  R m;
  switch (model) {
    case 1: m = hertz_mag(overlap, dot(rv, n), es, rs, ms, beta_abs); break;
    case 0: {
      R kn = es * rs;
      R gn = R(0.5) * sqrt(ms * kn);
      m = lsd_mag(overlap, dot(rv, n), kn, gn);
    } break;
    case 2: {
      R kn = es * rs;
      R vn = wall ? dot(rv, n) : dot(t3(R(0), R(0), R(0)), n);
      m = lsd_mag(overlap, vn, kn, R(0));
    } break;
    case 3: m = jkr_mag(overlap, es, rs, gamma); break;
    default: m = sjkr_mag(overlap, dot(rv, n), es, rs, gamma); break;
  }
  return m;
}
// The same with the normal relative speed given (vn = rv . n; the FP32 form
// forms it in FP64). The hysteretic particle-particle law keeps the
// reference's zero velocity.
template <typename R>
__device__ __forceinline__ R normal_mag_vn(int model, R overlap, T3<R> n, R vn, R es, R rs, R ms, R beta_abs,
                                          R gamma) {
  switch (model) {
    case 1: return hertz_mag(overlap, vn, es, rs, ms, beta_abs);
    case 0: {
      R kn = es * rs;
      R gn = R(0.5) * sqrt(ms * kn);
      return lsd_mag(overlap, vn, kn, gn);
    }
    case 2: return lsd_mag(overlap, dot(t3(R(0), R(0), R(0)), n), es * rs, R(0));
    case 3: return jkr_mag(overlap, es, rs, gamma);
    default: return sjkr_mag(overlap, vn, es, rs, gamma);
  }
}
// The vector form, f n, as the reference returns it.
template <typename R>
__device__ __forceinline__ T3<R> normal_force(int model, R overlap, T3<R> n, T3<R> rv, R es, R rs, R ms, R beta_abs,
                                              R gamma, bool wall) {
  return normal_mag<R>(model, overlap, n, rv, es, rs, ms, beta_abs, gamma, wall) * n;
}

// src/physics.rs:385-397 (direction by one reciprocal square root)
template <typename R>
__device__ __forceinline__ T3<R> coulomb_force(R fn, T3<R> rv, T3<R> n, R mu) {
  T3<R> vt = rv - dot(rv, n) * n;
  const R vt2 = dot(vt, vt);
  if (vt2 < R(1e-8)) return t3(R(0), R(0), R(0));
  R inv = rsqrt(vt2);
  T3<R> dir = vt * inv;
  return (-mu * fn) * dir;
}
// Coulomb from a given tangential relative velocity vt = rv - (rv . n) n.
template <typename R>
__device__ __forceinline__ T3<R> coulomb_force_vt(R fn, T3<R> vt, R mu) {
  const R vt2 = dot(vt, vt);
  if (vt2 < R(1e-8)) return t3(R(0), R(0), R(0));
  return (-mu * fn) * (vt * rsqrt(vt2));
}
// src/physics.rs:400-434 with the spring `xi` in registers.
template <typename R>
__device__ __forceinline__ T3<R> spring_coulomb_vt(R fn, T3<R> vt, T3<R>& xi, R kt, R mu, R dt) {
  xi = xi + vt * dt;
  T3<R> trial = (-kt) * xi;
  R tm = len(trial);
  R fc = mu * fn;
  if (tm > fc) {
    T3<R> dir = tm > R(1e-6) ? trial / tm : t3(R(0), R(0), R(0));
    T3<R> ft = fc * dir;
    xi = (-ft) / kt;
    return ft;
  }
  return trial;
}
template <typename R>
__device__ __forceinline__ T3<R> spring_coulomb(R fn, T3<R> rv, T3<R> n, T3<R>& xi, R kt, R mu, R dt) {
  return spring_coulomb_vt(fn, rv - dot(rv, n) * n, xi, kt, mu, dt);
}

// One contact seen from particle i (src/simulation.rs:358-460), for a pair
// that passed the cutoff test. Inputs in FP64; the law arithmetic in R.
// Writes the contact force on i and its torque r_a x f in FP64 and returns
// true. In FP32 it returns false, touching nothing, when a discontinuous
// decision of the reference's laws (Coulomb's |v_t|^2 < 1e-8, sJKR's
// loading/unloading sign and detachment, JKR's cut-offs) or an sJKR
// near-cancellation lies within FP32 rounding: the caller then evaluates the
// pair in FP64, so both forms take the same branches.
// L holds the material constants of the pair's group. With P.jkr_solver != 0
// the JKR magnitude comes from jkr_learned (`guess` is the network's a/R*, or
// negative / NaN for none; `tally` counts accepted / zero / fallback / walk
// and FP32 Newton steps when not null). A pair that needs the reference's
// Newton iteration sets *deferred and returns at once, touching nothing, when
// `deferred` is given; `newton` forces the reference's iteration.
template <typename R, bool PHYS, bool HIST>
__device__ __forceinline__ bool pair_contact(const StepParams& P, const Law& L, V d, double d2, double rsum, double ri,
                                             double rj, double mi, double mj, V vi, V vj, V wi, V wj, double* hist,
                                             size_t plane, T3<R>& fc_out, T3<R>& tc_out, T3<R>& n_out,
                                             bool& excess,
                                             float guess = -1.0f, uint32_t* tally = nullptr,
                                             bool* deferred = nullptr, bool newton = false) {
  constexpr bool F32 = sizeof(R) == sizeof(float);
  R overlap;
  T3<R> n;
  V nd;         // the unit normal in FP64 (FP32 form: to ~1e-14, for the relative velocity below)
  double ovd;   // the overlap in FP64 (FP32 form: to ~1e-14 of r_sum)
  if (sizeof(R) == sizeof(double)) {
    const double dist = sqrt(d2);
    overlap = (R)(rsum - dist);
    ovd = (double)overlap;
    const double inv = 1.0 / dist;
    const V nd = dist > 1e-6 ? d * inv : vmk(0.0, 1.0, 0.0);
    n = cvt<R>(nd);
  } else {
    bool far_enough;
    if (d2 > 1.001e-12) far_enough = true;
    else if (d2 < 0.999e-12) far_enough = false;
    else far_enough = sqrt(d2) > 1e-6;  // exact FP64 decision near the threshold
    if (far_enough) {
      // 1/|d| from the FP32 reciprocal square root and one FP64 Newton step
      // (relative error ~1e-14, no FP64 square root or division); |d| is
      // d^2 times it. The overlap is then good to ~1e-14 of r_sum: the JKR
      // contact radius next to its fold and the damping of a grazing contact
      // are sensitive to it.
      const double r0 = (double)rsqrtf((float)d2);
      const double inv = r0 * (1.5 - (0.5 * d2) * (r0 * r0));
      ovd = rsum - d2 * inv;
      nd = d * inv;
      n = cvt<R>(nd);
    } else {
      ovd = rsum - sqrt(d2);
      nd = vmk(0.0, 1.0, 0.0);
      n = t3(R(0), R(1), R(0));
    }
    overlap = (R)ovd;
  }
  const R rir = (R)ri, rjr = (R)rj;
  if (overlap > R(0.2) * fmin(rir, rjr)) excess = true;
  const T3<R> ra = (-n) * rir;
  const T3<R> rb = n * rjr;
  T3<R> rv, vt;
  R vn;
  if (sizeof(R) == sizeof(double)) {
    const T3<R> va = cvt<R>(vi) + cross(cvt<R>(wi), ra);
    const T3<R> vb = cvt<R>(vj) + cross(cvt<R>(wj), rb);
    rv = va - vb;
    vn = dot(rv, n);
    vt = rv - vn * n;
  } else {
    // In a rolling or sticking contact, and along the normal, the relative
    // velocity at the contact point is a small difference of large terms
    // (the spin terms w x r): rounded in FP32 they would swamp the normal
    // speed of the damping and the slip direction of the friction. So it is
    // formed in FP64, as (v_i - v_j) - (w_i r_i + w_j r_j) x n (the same
    // quantity as va - vb with r_a = -n r_i, r_b = n r_j), and only then
    // rounded for the FP32 laws.
    // Its normal part (the damping's speed) and tangential part (the slip)
    // are split in FP64 too: in a sliding contact the normal speed is a
    // small remainder of |rv|, in a head-on one the slip is.
    const V W = wi * ri + wj * rj;
    const V rvd = (vi - vj) - cross(W, nd);
    const double vnd = dot(rvd, nd);
    rv = cvt<R>(rvd);
    vn = (R)vnd;
    vt = cvt<R>(rvd - vnd * nd);
  }
  const R rs = (rir * rjr) / (rir + rjr);
  const R ms = ((R)mi * (R)mj) / ((R)mi + (R)mj);
  R fmag;
  int jkind = JKR_FALLBACK;
  if (P.nmodel == 3 && P.jkr_solver != 0 && !newton && L.gamma_pp > 0.0) {
    double fmd = 0.0;
    uint32_t it = 0;
    jkind = jkr_learned(P, L, ovd, (double)rs, guess, fmd, it);
    if (jkind != JKR_FALLBACK) fmag = (R)fmd;
    if (tally) {
      tally[jkind == JKR_CONVERGES ? 0 : (jkind == JKR_ZERO ? 1 : (jkind == JKR_WALK ? 5 : 2))] += 1;
      tally[4] += it;
    }
    if (jkind == JKR_FALLBACK && deferred) {
      *deferred = true;
      return true;
    }
  }
  if (jkind != JKR_FALLBACK) {
  } else if (F32 && P.nmodel == 3) {
    // The contact radius has a square-root fold next to the pull-off: there
    // the FP32 iteration cannot resolve the root (an FP32 residual moves it by
    // ~sqrt(1e-7) relative) and the pair is evaluated in FP64. Elsewhere the
    // certificates bound the slope away from zero.
    if (L.gamma_pp > 0.0) {
      const float x = (float)overlap / (float)rs, c = L.jkr_Cf / (float)rs;
      if (jkr_certify(x, c, jkr_c23(c), overlap > R(0)) == JKR_FALLBACK) return false;
    }
    bool near = false;
    fmag = jkr_mag<R>(overlap, (R)L.es_pp, rs, (R)L.gamma_pp, &near);
    if (near) return false;
  } else {
    fmag = normal_mag_vn<R>(P.nmodel, overlap, n, vn, (R)L.es_pp, rs, ms, (R)L.beta_abs, (R)L.gamma_pp);
  }
  if (F32 && P.nmodel == 4 && L.gamma_pp > 0.0) {
    const R gamma = (R)L.gamma_pp, es = (R)L.es_pp;
    const R f_pull = R(1.5) * R(kPi) * gamma * rs;
    const R delta_c = -sqrt(R(3) * (R(kPi) * R(kPi)) * (gamma * gamma) * rs / (es * es));
    if (fabs(vn) <= R(1e-6) * (len(rv) + R(1e-30))) return false;
    if (fabs(overlap - delta_c) <= R(1e-5) * fabs(delta_c)) return false;
    if (vn > R(0) && fabs(fmag) <= R(0.05) * f_pull) return false;
  }
  // |f n| = |f| for the unit normal (the reference takes the vector length)
  const T3<R> fnv = fmag * n;
  const R fnm = fabs(fmag);
  T3<R> ft;
  bool ft_zero = false;  // ft is +0: F = fn + 0 without the additions
  if (P.tmodel == 0) {
    if (F32) {
      const R vt2 = dot(vt, vt);
      if (fabs(vt2 - R(1e-8)) <= R(1e-5) * (vt2 + R(1e-8))) return false;
      ft = coulomb_force_vt<R>(fnm, vt, (R)L.mu);
    } else {
      ft = coulomb_force<R>(fnm, rv, n, (R)L.mu);
    }
  } else if (!PHYS) {
    // G* = 0 in parity mode (src/material.rs:39-50): the spring force is
    // 0 * (...), +-0, or NaN when Mindlin's sqrt(R* delta) is NaN or infinite
    // (a negative overlap); decided without the square root. With +0 for
    // the spring, F = fn + 0 is fn with -0 made +0.
    const R y = P.tmodel == 2 ? rs * overlap : rs;
    const R big = sizeof(R) == sizeof(float) ? R(FLT_MAX) : R(DBL_MAX);
    const bool finite = P.tmodel == 2 ? (y >= R(0) && y <= big) : (fabs(y) <= big);
    if (finite) {
      ft_zero = true;
      ft = t3(R(0), R(0), R(0));
    } else {
      const R nan = sizeof(R) == sizeof(float) ? (R)__int_as_float(0x7fc00000)
                                               : (R)__longlong_as_double(0x7ff8000000000000ll);
      ft = t3(nan, nan, nan);
    }
  } else {
    T3<R> xi_s = t3(R(0), R(0), R(0));
    if (overlap > R(0)) {
      R kt = P.tmodel == 2 ? R(8) * (R)L.gs_pp * sqrt(rs * overlap) : (R)L.gs_pp * rs;
      if (HIST) xi_s = t3((R)hist[0], (R)hist[plane], (R)hist[2 * plane]);
      xi_s = xi_s - dot(xi_s, n) * n;
      ft = F32 ? spring_coulomb_vt<R>(fnm, vt, xi_s, kt, (R)L.mu, (R)P.dt)
               : spring_coulomb<R>(fnm, rv, n, xi_s, kt, (R)L.mu, (R)P.dt);
    } else {
      ft = t3(R(0), R(0), R(0));
    }
    if (HIST) {
      hist[0] = (double)xi_s.x;
      hist[plane] = (double)xi_s.y;
      hist[2 * plane] = (double)xi_s.z;
    }
  }
  const T3<R> fc = ft_zero ? t3(plus_zero(fnv.x), plus_zero(fnv.y), plus_zero(fnv.z)) : fnv + ft;
  const T3<R> tc = cross(ra, fc);
  fc_out = fc;
  tc_out = tc;
  n_out = n;
  return true;
}

// Kahan-compensated s += d with residual r (src/particle.rs:12-18 and the
// reference's integrator): y = d - r, t = s + y, r = (t - s) - y, s = t.
__device__ __forceinline__ void kahan_add(V& s, V& r, V d) {
  const V y = d - r;
  const V t = s + y;
  r = (t - s) - y;
  s = t;
}

// Second half of velocity Verlet for one particle (src/simulation.rs:541-561):
// Kahan-compensated v += a dt/2 and omega += (tau/I) dt/2, I = 0.4 m r^2
// (tau/I as tau * (1/I), 1/I stored per particle in Bank::wres[k].w when the
// state is uploaded; v and x are unchanged).
__device__ __forceinline__ void second_half_kick(V& v, V& vres, V& w, V& wres, V a, V tau, double inv_inertia,
                                                 double dt) {
  const double hdt = 0.5 * dt;  // (0.5 a) dt == a (0.5 dt), both one rounding of a dt / 2
  V dv = a * hdt;
  V yv = dv - vres;
  V tv = v + yv;
  vres = (tv - v) - yv;
  v = tv;
  V aa = tau * inv_inertia;
  V dw = aa * hdt;
  V yw = dw - wres;
  V tw = w + yw;
  wres = (tw - w) - yw;
  w = tw;
}

// ------------------------------------------------------------- first half
// The force kernel only writes a and tau: neighbours read v and omega while
// it runs, so the second half kick of step n-1 is applied here, at the start
// of step n (when Ctrl::pending says a step owes it), and by k_second_half at
// the end of a stepping call. Then src/simulation.rs:176-263: periodic wrap,
// out-of-bounds removal (marked dead here and compacted by the host later;
// removal changes no other particle's update), Kahan-compensated half kick +
// drift + angular half kick. Also records the reference-grid cell code and
// requests a list rebuild when a particle moved more than half the skin since
// the last build.
//
// KAHAN = false is the mixed form's integrator: the same velocity-Verlet
// halves in plain FP64 (v += a dt/2, x += v dt, omega += (tau/I) dt/2), with
// the reference's Kahan residuals neither read nor updated. From zero
// residuals one step gives the same bits as the compensated form; over many
// steps positions and velocities differ from it by FP64 rounding (about one
// ulp per step), far below the FP32 pair forces' 1e-5. With the previous
// step's second half kick pending, the two half kicks are one kick of a dt.
// It takes ~45 of the ~85 FP64-pipe instructions per particle and 128 of the
// 484 bytes (the residuals' read and three writes) off this kernel.
template <bool KAHAN>
__global__ void __launch_bounds__(256) k_first_half(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const bool FUSE = C->pending != 0;
  const Bank B = P.bank[C->bank];
  const double dt = P.dt;
  const bool anyp = P.periodic[0] | P.periodic[1] | P.periodic[2];
  const float half_skin = (float)(0.5 * P.skin);
  // (0.5 a) dt and a (0.5 dt) are the same correctly rounded product
  const double hdt = 0.5 * dt;
  const float bminf[3] = {(float)P.bmin[0], (float)P.bmin[1], (float)P.bmin[2]};
  const float inv_hf = (float)P.inv_href;
  bool want_rebuild = false;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t fl = B.flags[k];
    if (fl & PF_DEAD) continue;
    D4 xr = B.xr[k], vm = B.vm[k], wc = B.wc[k];
    V x = xyz(xr), v = xyz(vm), w = xyz(wc);
    const bool moving = !(fl & PF_FIXED);
    V vres = vmk(0.0, 0.0, 0.0), wres = vres, xres = vres, dv = vres, dw = vres;
    double inv_inertia = 0.0, inv_mass = 0.0;
    if (moving) {
      // the fused second half of the previous step and this step's first
      // half kick with the same a and tau: the increments are computed once
      const V a = xyz(B.acc[k]);
      const V tau = xyz(B.tq[k]);
      const D4 vr4 = B.vres[k];
      inv_mass = vr4.w;
      const D4 wr4 = B.wres[k];
      inv_inertia = wr4.w;
      if (KAHAN) {
        vres = xyz(vr4);
        wres = xyz(wr4);
        xres = xyz(B.xres[k]);
      }
      // the mixed form joins the pending second half kick and this step's
      // first half kick into one kick of a dt
      const double kdt = (!KAHAN && FUSE) ? dt : hdt;
      dv = a * kdt;
      dw = KAHAN ? (tau * inv_inertia) * kdt : tau * (inv_inertia * kdt);
      if (KAHAN && FUSE) {
        kahan_add(v, vres, dv);
        kahan_add(w, wres, dw);
      }
    }
    // the FP32 mirror of x (written with it) decides most wrap and removal
    // tests without the FP64 comparisons: inside the inner interval of an
    // axis, x needs no wrap (periodic) or is kept (open)
    const float4 xo = B.xf[k];
    const bool in0 = xo.x > P.inner_lo[0] && xo.x < P.inner_hi[0];
    const bool in1 = xo.y > P.inner_lo[1] && xo.y < P.inner_hi[1];
    const bool in2 = xo.z > P.inner_lo[2] && xo.z < P.inner_hi[2];
    if (anyp) {
      if (P.periodic[0] && !in0) { if (x.x < P.bmin[0]) x.x = x.x + P.bsize[0]; else if (x.x >= P.bmax[0]) x.x = x.x - P.bsize[0]; }
      if (P.periodic[1] && !in1) { if (x.y < P.bmin[1]) x.y = x.y + P.bsize[1]; else if (x.y >= P.bmax[1]) x.y = x.y - P.bsize[1]; }
      if (P.periodic[2] && !in2) { if (x.z < P.bmin[2]) x.z = x.z + P.bsize[2]; else if (x.z >= P.bmax[2]) x.z = x.z - P.bsize[2]; }
    }
    bool keep = (P.periodic[0] || in0 || (x.x >= P.bmin[0] - 1.0 && x.x <= P.bmax[0] + 1.0)) &&
                (P.periodic[1] || in1 || (x.y >= P.bmin[1] - 1.0)) &&
                (P.periodic[2] || in2 || (x.z >= P.bmin[2] - 1.0 && x.z <= P.bmax[2] + 1.0));
    if (!keep) {
      B.flags[k] = fl | PF_DEAD;
      const double nan = __longlong_as_double(0x7ff8000000000000ll);
      xr.x = nan; xr.y = nan; xr.z = nan;
      B.xr[k] = xr;
      B.xf[k] = make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                            (float)xr.w);
      atomicAdd(&C->removed, 1ull);
      continue;
    }
    if (moving) {
      if (KAHAN) {
        kahan_add(v, vres, dv);
        kahan_add(x, xres, v * dt);
        kahan_add(w, wres, dw);
        B.vres[k] = D4{vres.x, vres.y, vres.z, inv_mass};
        B.xres[k] = D4{xres.x, xres.y, xres.z, 0.0};
        B.wres[k] = D4{wres.x, wres.y, wres.z, inv_inertia};
      } else {
        v = v + dv;
        x = x + v * dt;
        w = w + dw;
      }
      B.vm[k] = D4{v.x, v.y, v.z, vm.w};
      wc.x = w.x; wc.y = w.y; wc.z = w.z;
    }
    const float4 xf = make_float4((float)x.x, (float)x.y, (float)x.z, (float)xr.w);
    if (P.mode == 0) {
      const int32_t c0 = ref_axis_fast(x.x, xf.x, P.bmin[0], bminf[0], P.href, P.inv_href, inv_hf);
      const int32_t c1 = ref_axis_fast(x.y, xf.y, P.bmin[1], bminf[1], P.href, P.inv_href, inv_hf);
      const int32_t c2 = ref_axis_fast(x.z, xf.z, P.bmin[2], bminf[2], P.href, P.inv_href, inv_hf);
      wc.w = __longlong_as_double((long long)pack_code(c0, c1, c2));
    }
    B.wc[k] = wc;
    B.xr[k] = D4{x.x, x.y, x.z, xr.w};
    B.xf[k] = xf;
    float4 r0 = B.xref[k];
    float ddx = xf.x - r0.x, ddy = xf.y - r0.y, ddz = xf.z - r0.z;
    if (P.periodic[0]) ddx -= P.bsizef[0] * rintf(ddx / P.bsizef[0]);
    if (P.periodic[1]) ddy -= P.bsizef[1] * rintf(ddy / P.bsizef[1]);
    if (P.periodic[2]) ddz -= P.bsizef[2] * rintf(ddz / P.bsizef[2]);
    float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
    if (!(d2 <= half_skin * half_skin)) want_rebuild = true;  // NaN (no build yet) also rebuilds
  }
  if (want_rebuild) C->rebuild = 1;
}

// Completes the last step of a stepping call (the pending second half);
// k_clear_pending then marks the state complete. KAHAN as in k_first_half.
template <bool KAHAN>
__global__ void __launch_bounds__(256) k_second_half(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt || !C->pending) return;
  const Bank B = P.bank[C->bank];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t fl = B.flags[k];
    if (fl & (PF_DEAD | PF_FIXED)) continue;
    D4 vm = B.vm[k], wc = B.wc[k];
    const D4 wr4 = B.wres[k], vr4 = B.vres[k];
    V v = xyz(vm), w = xyz(wc), vres = xyz(vr4), wres = xyz(wr4);
    if (KAHAN) {
      second_half_kick(v, vres, w, wres, xyz(B.acc[k]), xyz(B.tq[k]), wr4.w, P.dt);
      B.vres[k] = D4{vres.x, vres.y, vres.z, vr4.w};
      B.wres[k] = D4{wres.x, wres.y, wres.z, wr4.w};
    } else {
      const double hdt = 0.5 * P.dt;
      v = v + xyz(B.acc[k]) * hdt;
      w = w + (xyz(B.tq[k]) * wr4.w) * hdt;
    }
    B.vm[k] = D4{v.x, v.y, v.z, vm.w};
    B.wc[k] = D4{w.x, w.y, w.z, wc.w};
  }
}

// Wall contacts of one particle (src/simulation.rs:464-523): the triangles
// listed in the triangle-grid cell of its centre, in mesh order.
// The cell lookup runs in FP32 on the position mirror (the host grows every
// triangle's box by a margin covering the FP32 error), and a triangle whose
// plane is farther than the radius (plus rounding) cannot touch the sphere,
// because the closest point lies in that plane: both skip FP64 work only.
// Triangles of another group than the particle's (gi) are not walls for it.

// The triangle-grid cell of an FP32 position: its range of triangle entries,
// or false outside the grid.
__device__ __forceinline__ bool tri_cell_range(const StepParams& P, float4 xf, uint32_t& s, uint32_t& e) {
  const float q0 = floorf((xf.x - P.tminf[0]) * P.tinvf);
  const float q1 = floorf((xf.y - P.tminf[1]) * P.tinvf);
  const float q2 = floorf((xf.z - P.tminf[2]) * P.tinvf);
  if (!(q0 >= 0.f && q1 >= 0.f && q2 >= 0.f && q0 < (float)P.tdims[0] && q1 < (float)P.tdims[1] &&
        q2 < (float)P.tdims[2]))
    return false;
  const uint32_t cell = (uint32_t)q0 + (uint32_t)P.tdims[0] * ((uint32_t)q1 + (uint32_t)P.tdims[1] * (uint32_t)q2);
  s = P.tstart[cell];
  e = P.tstart[cell + 1];
  return true;
}

// FP32 pretest of a sphere (centre xf, radius rf = xf.w, largest |coordinate|
// xmag, group gi) against a triangle: false when it cannot touch it.
__device__ __forceinline__ bool wall_pretest(const TriRec& tr, uint32_t gi, float4 xf, float xmag) {
  if (tr.group != GROUP_ALL && tr.group != gi) return false;
  const float rf = xf.w;
  // FP32 rounding of n, n.v0 and x moves n.x - n.v0 by at most
  // ~3e-7 (|x| + |n.v0|) + 1.1e-7 |x - v0|; the margin is larger
  const float4 pl = tr.plane;
  const float hd = fabsf(pl.x * xf.x + pl.y * xf.y + pl.z * xf.z - pl.w);
  const float mrg = 1e-6f * (1.0f + xmag + fabsf(pl.w) + rf) + 2e-7f * (xmag + tr.bound.x);
  if (hd > rf + mrg) return false;
  // the distance to the triangle is at least sqrt(hd^2 + s^2), s the
  // largest outward in-plane distance to an edge line (each with the
  // plane test's rounding margin; |m.v| <= sqrt(3) bound)
  const float4 g0 = tr.edge[0], g1 = tr.edge[1], g2 = tr.edge[2];
  const float s = fmaxf(fmaxf(g0.x * xf.x + g0.y * xf.y + g0.z * xf.z - g0.w,
                              g1.x * xf.x + g1.y * xf.y + g1.z * xf.z - g1.w),
                        g2.x * xf.x + g2.y * xf.y + g2.z * xf.z - g2.w);
  const float me = mrg + 4e-7f * tr.bound.x;
  const float hl = fmaxf(hd - mrg, 0.0f), sl = fmaxf(s - me, 0.0f);
  return !(hl * hl + sl * sl > rf * rf * (1.0f + 1e-6f));
}

// The FP64 contact of a sphere with a triangle that passed the pretest:
// force fc and torque r_a x fc on the sphere, or false (outputs untouched)
// when it does not touch the triangle.
__device__ __forceinline__ bool wall_contact(const StepParams& P, const Law& L, const TriRec& tr, V xi, V vi, V wi,
                                             double ri, double mi, V& fc_out, V& tc_out, bool& excess) {
  // closest point, src/mesh.rs:45-117 (same regions and clamps)
  const V v0 = vmk(tr.v0[0] - xi.x, tr.v0[1] - xi.y, tr.v0[2] - xi.z);
  const V e0 = vmk(tr.e0[0], tr.e0[1], tr.e0[2]), e1 = vmk(tr.e1[0], tr.e1[1], tr.e1[2]);
  const double a = tr.a, b = tr.b, c = tr.c, det = tr.det;
  const double dd = dot(e0, v0), ee = dot(e1, v0);
  const double s0 = b * ee - c * dd, t0 = b * dd - a * ee;
  double sc = s0, tc = t0;
  if (s0 + t0 < det) {
    if (s0 < 0.0) {
      if (t0 < 0.0) {
        if (dd < 0.0) { sc = fmin(fmax(-dd, 0.0), a); tc = 0.0; }
        else { sc = 0.0; tc = fmin(fmax(-ee, 0.0), c); }
      } else { sc = 0.0; tc = fmin(fmax(-ee, 0.0), c); }
    } else if (t0 < 0.0) {
      sc = fmin(fmax(-dd, 0.0), a); tc = 0.0;
    } else {
      const double inv = 1.0 / det;
      sc = sc * inv; tc = tc * inv;
    }
  } else {
    if (s0 < 0.0) {
      const double tmp0 = b + dd, tmp1 = c + ee;
      if (tmp1 > tmp0) {
        const double numer = tmp1 - tmp0;
        sc = numer / tr.denom; sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc); tc = 1.0 - sc;
      } else { tc = fmin(fmax(-ee, 0.0), c); sc = 0.0; }
    } else if (t0 < 0.0) {
      if (a + dd > b + ee) {
        const double numer = c + ee - b - dd;
        sc = numer / tr.denom; sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc); tc = 1.0 - sc;
      } else { sc = fmin(fmax(-ee, 0.0), c); tc = 0.0; }
    } else {
      const double numer = c + ee - b - dd;
      sc = numer / tr.denom; sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc); tc = 1.0 - sc;
    }
  }
  const V cp = vmk(tr.v0[0], tr.v0[1], tr.v0[2]) + sc * e0 + tc * e1;
  const V dv = xi - cp;
  const double dsq = dot(dv, dv);
  if (!(dsq < ri * ri)) return false;
  const double dist = sqrt(dsq);
  const double pen = ri - dist;
  const V n = dist > 1e-6 ? dv / dist : vmk(tr.n[0], tr.n[1], tr.n[2]);
  if (pen > 0.2 * ri) excess = true;
  const V ra = (-n) * ri;
  V rv = vi + cross(wi, ra);
  if (tr.motion != NO_MOTION) {  // a moving wall: relative to its surface velocity at the contact point
    const WallMotion& M = P.motions[tr.motion];
    const V vw = vmk(M.v[0], M.v[1], M.v[2]) + cross(vmk(M.w[0], M.w[1], M.w[2]), cp - vmk(M.c[0], M.c[1], M.c[2]));
    rv = rv - vw;
  }
  const V fnv = normal_force<double>(P.nmodel, pen, n, rv, L.es_pw, ri, mi, L.beta_abs, L.gamma_pw, true);
  const V fc = fnv + coulomb_force<double>(len(fnv), rv, n, L.mu);
  fc_out = fc;
  tc_out = cross(ra, fc);
  return true;
}

// All wall contacts of one particle in mesh order.
__device__ __forceinline__ void wall_forces(const StepParams& P, const Law& L, uint32_t gi, V xi, float4 xf, V vi,
                                            V wi, double ri, double mi, V& F, V& T, bool& excess) {
  uint32_t s, e;
  if (P.ntri == 0 || !tri_cell_range(P, xf, s, e)) return;
  const float xmag = fmaxf(fmaxf(fabsf(xf.x), fabsf(xf.y)), fabsf(xf.z));
  for (uint32_t t = s; t < e; ++t) {
    const TriRec& tr = P.tri[P.titems[t]];
    if (!wall_pretest(tr, gi, xf, xmag)) continue;
    V fc, tc;
    if (wall_contact(P, L, tr, xi, vi, wi, ri, mi, fc, tc, excess)) {
      F = F + fc;
      T = T + tc;
    }
  }
}

// ---------------------------------------------------------------- forces
// One thread per slot gathers its Verlet list: the exact FP64 cutoff test of
// src/simulation.rs:327-357, the reference's visit count in parity mode, the
// pair laws of src/simulation.rs:358-460 (in R), the wall triangles of
// src/simulation.rs:464-523 from the triangle grid, then a = g + F/m and
// tau = T (src/simulation.rs:265-271, 532-536). v and omega are only read.
template <bool PHYS, bool HIST, typename R>
__global__ void __launch_bounds__(128) k_force(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  const bool adh = (P.nmodel == 3 || P.nmodel == 4);
  const size_t plane = (size_t)P.n * P.cap;
  bool excess = false;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    const uint32_t fl = B.flags[k];
    if (fl & PF_DEAD) continue;
    const Law lw = law_of(P, B, k);
    const uint32_t gi = P.ngroups > 1 ? B.grp[k] : 0u;
    const D4 xi4 = B.xr[k], vi4 = B.vm[k], wi4 = B.wc[k];
    const V xi = xyz(xi4), vi = xyz(vi4), wi = xyz(wi4);
    const double ri = xi4.w, mi = vi4.w;
    const unsigned long long ci = (unsigned long long)__double_as_longlong(wi4.w);
    V F = vmk(0.0, 0.0, 0.0), T = vmk(0.0, 0.0, 0.0);
    const uint32_t cnt = B.ncnt[k];
    const uint32_t* row = B.nbr + (size_t)k * P.cap;
    unsigned long long hm = 0ull;  // springs this row writes (the live-spring mask)
    const float4 xif = B.xf[k];
    const float Xi = fmaxf(fmaxf(fabsf(xif.x), fabsf(xif.y)), fabsf(xif.z));
    for (uint32_t m = 0; m < cnt; ++m) {
      const uint32_t j = row[m];
      if (P.pretest) {
        // FP32 pretest on the position mirror: with u = 2^-24, each FP32
        // difference is within e = u (2X + 2 cut + L) of the FP64 one when the
        // pair is inside the cutoff, so d2f <= cut^2 + 3.47 e cut + 3 e^2 +
        // 12 u cut^2 there. Beyond the (larger) band below the pair is
        // certainly outside and the exact FP64 test is skipped.
        const float4 xjf = B.xf[j];
        float fx = xif.x - xjf.x, fy = xif.y - xjf.y, fz = xif.z - xjf.z;
        if (P.periodic[0]) { const float L = P.bsizef[0]; if (fx > 0.5f * L) fx -= L; else if (fx < -0.5f * L) fx += L; }
        if (P.periodic[1]) { const float L = P.bsizef[1]; if (fy > 0.5f * L) fy -= L; else if (fy < -0.5f * L) fy += L; }
        if (P.periodic[2]) { const float L = P.bsizef[2]; if (fz > 0.5f * L) fz -= L; else if (fz < -0.5f * L) fz += L; }
        const float d2f = fx * fx + fy * fy + fz * fz;
        const float rsf = xif.w + xjf.w;
        const float cutf = adh ? rsf * 1.5f : rsf;
        const float X = fmaxf(Xi, fmaxf(fmaxf(fabsf(xjf.x), fabsf(xjf.y)), fabsf(xjf.z)));
        const float e = 6.0e-8f * (2.0f * X + 2.0f * cutf + P.lmax);
        const float band = 4.1f * cutf * e + 3.0f * e * e + 1.0e-6f * cutf * cutf;
        if (d2f > cutf * cutf + band) {
          const size_t hi = (size_t)k * P.cap + m;
          if (HIST) {
            B.hist[hi] = 0.0;
            B.hist[plane + hi] = 0.0;
            B.hist[2 * plane + hi] = 0.0;
          }
          if (P.debug) P.dbgMult[hi] = 0;
          continue;
        }
      }
      const D4 xj4 = B.xr[j];
      V d = xi - xyz(xj4);
      if (P.periodic[0]) { if (d.x > P.bsize[0] * 0.5) d.x = d.x - P.bsize[0]; else if (d.x < -P.bsize[0] * 0.5) d.x = d.x + P.bsize[0]; }
      if (P.periodic[1]) { if (d.y > P.bsize[1] * 0.5) d.y = d.y - P.bsize[1]; else if (d.y < -P.bsize[1] * 0.5) d.y = d.y + P.bsize[1]; }
      if (P.periodic[2]) { if (d.z > P.bsize[2] * 0.5) d.z = d.z - P.bsize[2]; else if (d.z < -P.bsize[2] * 0.5) d.z = d.z + P.bsize[2]; }
      const double d2 = dot(d, d);
      const double rj = xj4.w;
      const double rsum = ri + rj;
      const double margin = adh ? rsum * 0.5 : 0.0;
      const double cut = rsum + margin;
      int visits = 0;
      const size_t hi = (size_t)k * P.cap + m;
      if (d2 < cut * cut) {
        const D4 wj4 = B.wc[j];
        visits = PHYS ? 1 : ref_visits(P, ci, (unsigned long long)__double_as_longlong(wj4.w));
        if (visits > 0) {
          const D4 vj4 = B.vm[j];
          V fc, tc, nrm;
          T3<R> fr, tr, nr;
          if (pair_contact<R, PHYS, HIST>(P, lw, d, d2, rsum, ri, rj, mi, vj4.w, vi, xyz(vj4), wi, xyz(wj4),
                                          HIST ? B.hist + hi : nullptr, plane, fr, tr, nr, excess)) {
            fc = cvt<double>(fr);
            tc = cvt<double>(tr);
          } else {
            pair_contact<double, PHYS, HIST>(P, lw, d, d2, rsum, ri, rj, mi, vj4.w, vi, xyz(vj4), wi, xyz(wj4),
                                             HIST ? B.hist + hi : nullptr, plane, fc, tc, nrm, excess);
          }
          if (HIST && m < 64) hm |= 1ull << m;
          for (int t = 0; t < visits; ++t) {
            F = F + fc;
            T = T + tc;
          }
        }
      }
      if (HIST && visits == 0) {
        B.hist[hi] = 0.0;
        B.hist[plane + hi] = 0.0;
        B.hist[2 * plane + hi] = 0.0;
      }
      if (P.debug) P.dbgMult[hi] = (uint8_t)visits;
    }
    if (HIST && hm) B.hmask[k] |= hm;
    wall_forces(P, lw, gi, xi, xif, vi, wi, ri, mi, F, T, excess);
    if (P.debug) {
      P.dbgF[3 * (size_t)k] = F.x; P.dbgF[3 * (size_t)k + 1] = F.y; P.dbgF[3 * (size_t)k + 2] = F.z;
      P.dbgT[3 * (size_t)k] = T.x; P.dbgT[3 * (size_t)k + 1] = T.y; P.dbgT[3 * (size_t)k + 2] = T.z;
    }
    if (!isfinite(F.x + F.y + F.z + T.x + T.y + T.z)) atomicOr(&C->status, (unsigned)ST_NAN);
    // apply (src/simulation.rs:532-536), F/m as F (1/m) with 1/m stored per
    // particle; the second half kick of this step runs in the next
    // k_first_half or in k_second_half
    const V a = vmk(P.gravity[0], P.gravity[1], P.gravity[2]) + F * B.vres[k].w;
    const V tau = vmk(0.0, 0.0, 0.0) + T;
    B.acc[k] = D4{a.x, a.y, a.z, 0.0};
    B.tq[k] = D4{tau.x, tau.y, tau.z, 0.0};
  }
  if (excess) C->overlap_flag = 1;
}

// ------------------------------------------------- contact-parallel forces
// One thread per particle leaves every lane idle while a neighbour of another
// lane is in contact (measured: ~9 of 32 lanes active, FP64 pipe saturated).
// Here the per-particle pass only filters (FP32 pretest, exact FP64 cutoff,
// visit counts); the pair laws run one thread per pair, each pair once, and a
// last pass sums every particle's contact results in list order.

// FP32 pretest on the position mirror: with u = 2^-24, each FP32 difference
// is within e = u (2X + 2 cut + L) of the FP64 one when the pair is inside the
// cutoff, so d2f <= cut^2 + 3.47 e cut + 3 e^2 + 12 u cut^2 there; beyond the
// larger band below the pair is certainly outside the exact FP64 test.
__device__ __forceinline__ bool pretest_far(const StepParams& P, float4 xif, float Xi, float4 xjf, bool adh) {
  float fx = xif.x - xjf.x, fy = xif.y - xjf.y, fz = xif.z - xjf.z;
  if (P.periodic[0]) { const float L = P.bsizef[0]; if (fx > 0.5f * L) fx -= L; else if (fx < -0.5f * L) fx += L; }
  if (P.periodic[1]) { const float L = P.bsizef[1]; if (fy > 0.5f * L) fy -= L; else if (fy < -0.5f * L) fy += L; }
  if (P.periodic[2]) { const float L = P.bsizef[2]; if (fz > 0.5f * L) fz -= L; else if (fz < -0.5f * L) fz += L; }
  const float d2f = fx * fx + fy * fy + fz * fz;
  const float rsf = xif.w + xjf.w;
  const float cutf = adh ? rsf * 1.5f : rsf;
  const float X = fmaxf(Xi, fmaxf(fmaxf(fabsf(xjf.x), fabsf(xjf.y)), fabsf(xjf.z)));
  const float e = 6.0e-8f * (2.0f * X + 2.0f * cutf + P.lmax);
  const float band = 4.1f * cutf * e + 3.0f * e * e + 1.0e-6f * cutf * cutf;
  return d2f > cutf * cutf + band;
}

// Minimum image on the periodic axes. A difference whose magnitude has a
// smaller high word than bsize/4 is below bsize/4 (and NaN is not), so it
// needs no FP64 comparison.
__device__ __forceinline__ bool near_axis(double d, uint32_t q_hi) {
  return (uint32_t)(__double2hiint(d) & 0x7FFFFFFF) < q_hi;
}
__device__ __forceinline__ V mic(const StepParams& P, V d) {
  if (P.periodic[0] && !near_axis(d.x, P.bq_hi[0])) { if (d.x > P.bsize[0] * 0.5) d.x = d.x - P.bsize[0]; else if (d.x < -P.bsize[0] * 0.5) d.x = d.x + P.bsize[0]; }
  if (P.periodic[1] && !near_axis(d.y, P.bq_hi[1])) { if (d.y > P.bsize[1] * 0.5) d.y = d.y - P.bsize[1]; else if (d.y < -P.bsize[1] * 0.5) d.y = d.y + P.bsize[1]; }
  if (P.periodic[2] && !near_axis(d.z, P.bq_hi[2])) { if (d.z > P.bsize[2] * 0.5) d.z = d.z - P.bsize[2]; else if (d.z < -P.bsize[2] * 0.5) d.z = d.z + P.bsize[2]; }
  return d;
}

// Whether a JKR pair goes to the network queue: jkr_learned's certificate on
// the FP32 position mirror, its xi thresholds widened by the mirror's
// rounding (~2.4e-7 of the coordinates). A queued pair the exact test rejects
// only wastes a network row; a converging pair without a row falls back to the
// reference's Newton.
__device__ __forceinline__ bool jkr_net_hint(const StepParams& P, float Cf, float4 xif, float4 xjf) {
  float fx = xif.x - xjf.x, fy = xif.y - xjf.y, fz = xif.z - xjf.z;
  if (P.periodic[0]) { const float L = P.bsizef[0]; if (fx > 0.5f * L) fx -= L; else if (fx < -0.5f * L) fx += L; }
  if (P.periodic[1]) { const float L = P.bsizef[1]; if (fy > 0.5f * L) fy -= L; else if (fy < -0.5f * L) fy += L; }
  if (P.periodic[2]) { const float L = P.bsizef[2]; if (fz > 0.5f * L) fz -= L; else if (fz < -0.5f * L) fz += L; }
  const float rsum = xif.w + xjf.w;
  const float rs = xif.w * xjf.w / rsum;
  const float c = Cf / rs;
  if (!(c >= kJkrCMin && c <= kJkrCMax)) return false;
  const float c23 = jkr_c23(c);
  const float x = (rsum - sqrtf(fx * fx + fy * fy + fz * fz)) / rs;
  const float X = fmaxf(fmaxf(fmaxf(fabsf(xif.x), fabsf(xif.y)), fabsf(xif.z)),
                        fmaxf(fmaxf(fabsf(xjf.x), fabsf(xjf.y)), fabsf(xjf.z)));
  const float m = 0.02f + 2.4e-7f * (2.0f * X + rsum + P.lmax) / (rs * c23);
  const float xi = x / c23;
  if (xi < kJkrXiNeg - m) return false;
  if (xi > m && xi < kJkrXiPos - m) return false;
  const float f1 = logf(rs);
  if (f1 < P.jdom_lo[1] || f1 > P.jdom_hi[1]) return false;
  if (sqrtf(fmaxf(xi - m + kJkrKappa, 0.0f)) > P.jdom_hi[0]) return false;
  return true;
}

// Whether a JKR pair is certainly in the ZERO region of jkr_certify (no
// contact radius makes the reference's residual smaller than 1e-3 R*, so its
// JKR force is exactly zero), decided on the FP32 position mirror with that
// mirror's rounding added to the certificate's margin. Symmetric in (i, j)
// bit for bit, so both ends of a pair drop it or keep it together.
__device__ __forceinline__ bool jkr_far_zero(const StepParams& P, float Cf, float4 xif, float Xi, float4 xjf) {
  float fx = xif.x - xjf.x, fy = xif.y - xjf.y, fz = xif.z - xjf.z;
  if (P.periodic[0]) { const float L = P.bsizef[0]; if (fx > 0.5f * L) fx -= L; else if (fx < -0.5f * L) fx += L; }
  if (P.periodic[1]) { const float L = P.bsizef[1]; if (fy > 0.5f * L) fy -= L; else if (fy < -0.5f * L) fy += L; }
  if (P.periodic[2]) { const float L = P.bsizef[2]; if (fz > 0.5f * L) fz -= L; else if (fz < -0.5f * L) fz += L; }
  const float rsum = xif.w + xjf.w;
  const float rs = (xif.w * xjf.w) / rsum;
  const float c = Cf / rs;
  if (!(c > 0.0f && c < 1e30f)) return false;
  const float c23 = jkr_c23(c);
  const float d = sqrtf(fx * fx + fy * fy + fz * fz);
  const float X = fmaxf(Xi, fmaxf(fmaxf(fabsf(xjf.x), fabsf(xjf.y)), fabsf(xjf.z)));
  // per-axis FP32 difference error <= 6e-8 (2X + 2 cut + L) (as in pretest_far),
  // so |d_f - d| <= 1.8e-7 (2X + 3 r_sum + L) + 4e-7 d, radii rounded too
  const float e = (1.8e-7f * (2.0f * X + 3.0f * rsum + P.lmax) + 4e-7f * (d + rsum)) / rs;
  const float x = (rsum - d) / rs;
  return x + kJkrKappa * c23 + 1e-3f < -(1e-5f * (fabsf(x) + c23 + 1e-3f) + 2.0f * e);
}

// Whether an sJKR pair certainly has zero normal force: overlap below
// delta_c = -sqrt(3 pi^2 gamma^2 R* / E*^2) (src/physics.rs:234-325; with
// gamma <= 0 the law is Hertz's, zero for a negative overlap), decided on the
// FP32 mirror with its rounding (as jkr_far_zero) and 1e-5 of delta_c as
// margin. Symmetric in (i, j) bit for bit.
__device__ __forceinline__ bool sjkr_far_zero(const StepParams& P, const Law& L, float4 xif, float Xi, float4 xjf) {
  float fx = xif.x - xjf.x, fy = xif.y - xjf.y, fz = xif.z - xjf.z;
  if (P.periodic[0]) { const float Lp = P.bsizef[0]; if (fx > 0.5f * Lp) fx -= Lp; else if (fx < -0.5f * Lp) fx += Lp; }
  if (P.periodic[1]) { const float Lp = P.bsizef[1]; if (fy > 0.5f * Lp) fy -= Lp; else if (fy < -0.5f * Lp) fy += Lp; }
  if (P.periodic[2]) { const float Lp = P.bsizef[2]; if (fz > 0.5f * Lp) fz -= Lp; else if (fz < -0.5f * Lp) fz += Lp; }
  const float rsum = xif.w + xjf.w;
  const float rs = (xif.w * xjf.w) / rsum;
  const float d = sqrtf(fx * fx + fy * fy + fz * fz);
  const float X = fmaxf(Xi, fmaxf(fmaxf(fabsf(xjf.x), fabsf(xjf.y)), fabsf(xjf.z)));
  const float e = 1.8e-7f * (2.0f * X + 3.0f * rsum + P.lmax) + 4e-7f * (d + rsum);
  float dc = 0.0f;
  if (L.gamma_pp > 0.0) {
    const float g = (float)L.gamma_pp, es = (float)L.es_pp, pi = 3.14159265f;
    dc = -sqrtf(3.0f * (pi * pi) * (g * g) * rs / (es * es));
  }
  return (rsum - d) + e < dc - 1e-5f * fabsf(dc);
}

// Exclusive prefix of v over the lanes of the warp, and the warp's total.
// Every lane of the warp takes part.
__device__ __forceinline__ uint32_t warp_exclusive(uint32_t v, uint32_t& total) {
  const int lane = threadIdx.x & 31;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xFFFFFFFFu, x, 31);
  return x - v;
}

// v slots of the array behind a device counter for each lane of the warp,
// contiguous in lane order, with one atomic per warp: returns this lane's
// first slot. Every lane of the warp takes part.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* ctr, uint32_t v) {
  uint32_t total;
  const uint32_t ex = warp_exclusive(v, total);
  uint32_t base = 0;
  if ((threadIdx.x & 31) == 0 && total) base = atomicAdd(ctr, total);
  return __shfl_sync(0xFFFFFFFFu, base, 0) + ex;
}

// The contact pass's counters (records, evaluating records, network queue,
// deferred pairs, wall candidates) start every force pass at zero.
constexpr int CTOT_WORDS = 8;

// Pass 1 (FP32 and integer work only): the candidates of each particle, i.e.
// list entries the FP32 pretest cannot rule out and that the reference's loop
// visits from this end (visit counts from both ends recorded); marks the ones
// that evaluate their pair (the lower slot of a pair seen from both ends, or
// the only end that sees it). The pretest is symmetric, so a pair seen from
// both ends is a candidate at both. Each warp then reserves, with one atomic
// per counter, the result slots of its particles' records (coff) and their
// places in the compact list of evaluating records (and the network queue):
// where a record's result lands changes nothing in its value, and each
// particle's results stay contiguous and in list order. The block size is a
// multiple of 32 and every lane of a warp runs the same number of iterations.
template <bool PHYS, bool HIST>
__global__ void __launch_bounds__(256, 4) k_contact_filter(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  const bool adh = (P.nmodel == 3 || P.nmodel == 4);
  const bool learn_any = P.jkr_solver == 1 && P.nmodel == 3 && P.mlp != nullptr;
  // Certified-zero JKR pairs add exactly +-0 to F and T when the tangential
  // force then vanishes too (Coulomb with |F_n| = 0; physical-mode springs
  // reset out of contact): with the certified solvers they are not
  // candidates at all. Parity-mode springs (G* = 0, NaN for Mindlin at
  // negative overlap) and debug recording keep every pair.
  const bool zdrop_any = P.jkr_solver != 0 && P.nmodel == 3 && P.pretest && !P.debug && (P.tmodel == 0 || PHYS);
  // the same for sJKR, whose zero region is explicit (no iteration to certify)
  const bool sdrop = P.nmodel == 4 && P.pretest && !P.debug && (P.tmodel == 0 || PHYS);
  const size_t plane = (size_t)P.n * P.cap;
  // slots in the rebuild-time order (tiles of 256 sorted by list length), so
  // a warp's lanes walk lists of similar length
  for (int i0 = blockIdx.x * blockDim.x; i0 < P.n; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + (int)threadIdx.x;
    const int k = i < P.n ? (int)P.aorder[i] : -1;
    uint32_t nrec = 0, ncmp = 0, nnet = 0, nw = 0, ts = 0, te = 0, gi = 0;
    float4 xif = make_float4(0.f, 0.f, 0.f, 0.f);
    float Xi = 0.f;
    const uint32_t flk = k >= 0 ? B.flags[k] : PF_DEAD;
    if (!(flk & PF_DEAD)) {
      const unsigned long long ci = PHYS ? 0ull : (unsigned long long)__double_as_longlong(B.wc[k].w);
      // visits of a neighbour in the same reference cell (most pairs at a 1 m
      // cell): a constant, without the 27-cell walk of ref_visits
      const int same = (PHYS || !ref_inside(P, ci)) ? 0 : P.same_cell_visits;
      const Law lw = law_of(P, B, k);  // pairs never cross groups (the lists exclude them)
      const bool adhesive = lw.gamma_pp > 0.0;
      const bool learn = learn_any && adhesive, zdrop = zdrop_any && adhesive;
      xif = B.xf[k];
      Xi = fmaxf(fmaxf(fabsf(xif.x), fabsf(xif.y)), fabsf(xif.z));
      const uint32_t cnt = B.ncnt[k];
      const uint32_t* row = B.nbr + (size_t)k * P.cap;
      CRec* out = P.crec + (size_t)k * P.cap;
      unsigned long long hm = HIST ? B.hmask[k] : 0ull;
      const unsigned long long hm0 = hm;
      // the next two entries and their FP32 positions are loaded while this
      // one is tested (rows and positions are read-only during the pass)
      uint32_t jn = cnt > 0 ? __ldg(row) : 0u, jn2 = cnt > 1 ? __ldg(row + 1) : 0u;
      float4 xn = cnt > 0 ? __ldg(B.xf + jn) : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 xn2 = cnt > 1 ? __ldg(B.xf + jn2) : make_float4(0.f, 0.f, 0.f, 0.f);
      for (uint32_t m = 0; m < cnt; ++m) {
        const uint32_t j = jn;
        const float4 xjf = xn;
        jn = jn2;
        xn = xn2;
        if (m + 2 < cnt) {
          jn2 = __ldg(row + m + 2);
          xn2 = __ldg(B.xf + jn2);
        }
        const size_t hi = (size_t)k * P.cap + m;
        int vij = 0, vji = 0;
        if (!(P.pretest && pretest_far(P, xif, Xi, xjf, adh)) && !(zdrop && jkr_far_zero(P, lw.jkr_Cf, xif, Xi, xjf)) &&
            !(sdrop && sjkr_far_zero(P, lw, xif, Xi, xjf))) {
          if (PHYS) {
            vij = vji = 1;
          } else {
            const unsigned long long cj = (unsigned long long)__double_as_longlong(B.wc[j].w);
            if (cj == ci) {
              vij = vji = same;
            } else {
              vij = ref_visits(P, ci, cj);
              vji = ref_visits(P, cj, ci);
            }
          }
        }
        if (vij > 0) {
          const bool evaluates = !(vji > 0 && (uint32_t)k > j);
          const uint32_t net = (learn && evaluates && jkr_net_hint(P, lw.jkr_Cf, xif, xjf)) ? CREC_NET : 0u;
          out[nrec] = CRec{j, m | ((uint32_t)vij << 16) | ((uint32_t)vji << 24) | net};
          ++nrec;
          if (evaluates) ++ncmp;
          if (net) ++nnet;
        } else {
          // a spring out of reach resets; one already +0 (its bit clear) stays
          if (HIST && (m >= 64 || ((hm >> m) & 1ull))) {
            B.hist[hi] = 0.0;
            B.hist[plane + hi] = 0.0;
            B.hist[2 * plane + hi] = 0.0;
            if (m < 64) hm &= ~(1ull << m);
          }
          if (P.debug) P.dbgMult[hi] = 0;
        }
      }
      if (HIST && hm != hm0) B.hmask[k] = hm;
      // wall candidates: the triangles of its triangle-grid cell that pass
      // the FP32 pretest, counted here and listed once the arena is reserved
      if (P.ntri > 0 && !(P.wall_far_ok && (flk & PF_WALLFAR)) && tri_cell_range(P, xif, ts, te)) {
        gi = P.ngroups > 1 ? B.grp[k] : 0u;
        for (uint32_t t = ts; t < te; ++t) nw += wall_pretest(P.tri[P.titems[t]], gi, xif, Xi) ? 1u : 0u;
      }
    }
    __syncwarp();
    const uint32_t rb = warp_reserve(P.ctot, nrec);
    uint32_t q = warp_reserve(P.ctot + 1, ncmp);
    uint32_t qn = learn_any ? warp_reserve(P.ctot + 2, nnet) : 0u;
    const uint32_t wb = P.ntri > 0 ? warp_reserve(P.ctot + 4, nw) : 0u;
    if (k < 0) continue;
    P.ccnt[k] = nrec;
    P.coff[k] = rb;
    if (P.ntri > 0) {
      if (nw > 0 && wb + nw <= P.wcap) {  // in mesh order, as the reference visits them
        uint2* dst = P.warena + wb;
        uint32_t c = 0;
        for (uint32_t t = ts; t < te && c < nw; ++t) {
          const uint32_t id = P.titems[t];
          if (wall_pretest(P.tri[id], gi, xif, Xi)) dst[c++] = make_uint2((uint32_t)k, id);
        }
      } else if (nw > 0) {  // the arena is full: the step halts and the host grows it
        atomicMax(&C->wall_need, wb + nw);
        atomicOr(&C->halt, HALT_WALLS);
      }
      P.wcnt[k] = nw;
      P.woff[k] = wb;
    }
    if (ncmp == 0) continue;
    // the evaluating records into the compact list (the queued ones into the
    // network queue too), read back from the row this thread just wrote
    const size_t base = (size_t)k * P.cap;
    const CRec* out = P.crec + base;
    for (uint32_t c = 0; c < nrec; ++c) {
      const CRec r = out[c];
      if (!(crec_vji(r.mv) > 0 && (uint32_t)k > r.j)) {
        if (r.mv & CREC_NET) P.jq[qn++] = make_uint2(q, (uint32_t)(base + c));
        P.clist[q++] = (uint32_t)(base + c);
      }
    }
  }
}

// Pass 2b: the JKR network over the queue, 32 pairs per warp on the tensor
// cores (weights staged once per block in shared memory). Features from the
// FP64 positions: the overlap from r_sum^2 - d^2 in FP64, the rest in FP32.
// Writes the predicted a/R* of each queued pair, NaN outside the training
// range.
__global__ void __launch_bounds__(128) k_jkr_mlp(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const uint32_t qn = P.ctot[2];
  if ((uint32_t)blockIdx.x * blockDim.x >= qn) return;
  __shared__ MlpInfer M;
  {
    const uint4* src = reinterpret_cast<const uint4*>(P.mlp);
    uint4* dst = reinterpret_cast<uint4*>(&M);
    for (int i = threadIdx.x; i < (int)(sizeof(MlpInfer) / 16); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const Bank B = P.bank[C->bank];
  const int lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < qn; base += stride) {
    const uint32_t idx = base + lane;
    const bool valid = idx < qn;
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    float ub = 0.f;
    bool ok = false;
    uint32_t q = 0;
    if (valid) {
      const uint2 it = P.jq[idx];
      q = it.x;
      const uint32_t s = it.y;
      const uint32_t k = s / (uint32_t)P.cap;
      const uint32_t j = P.crec[s].j;
      const D4 xi4 = B.xr[k], xj4 = B.xr[j];
      const V d = mic(P, xyz(xi4) - xyz(xj4));
      const double d2 = dot(d, d);
      const double rsum = xi4.w + xj4.w;
      const float ov = (float)(rsum * rsum - d2) / ((float)rsum + sqrtf((float)d2));
      const float rs = ((float)xi4.w * (float)xj4.w) / (float)rsum;  // a feature: FP32 is enough
      const float x = ov / rs;
      const Law lw = law_of(P, B, (int)k);
      const float c = lw.jkr_Cf / rs;
      const float c23 = jkr_c23(c);
      float raw[4];
      jkr_raw_features(x, c23, rs, (float)lw.es_pp, (float)lw.gamma_pp, raw);
      ok = true;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        ok = ok && raw[a] >= P.jdom_lo[a] && raw[a] <= P.jdom_hi[a];
        f[a] = (raw[a] - M.xmean[a]) * M.xinv[a];
      }
      ub = jkr_ubase(x, c23);
    }
    const float y = mlp_forward_warp(&M, f);
    if (valid) P.jguess[q] = ok ? __expf(y * M.ystd + M.ymean) * ub : __int_as_float(0x7FC00000);
  }
}

// Pass 3: one thread per candidate pair: the exact FP64 cutoff test of
// src/simulation.rs:343-357, then the pair laws. The force on the row's
// particle times its visit count goes to its result; the other end receives
// exactly the negated force (the reference's formula is sign-symmetric:
// evaluated from that end it gives -f bit for bit) times its own visit count,
// with its own torque (n r_j) x (-f), and in physical mode the negated spring.
// A candidate outside the cutoff gives zero results at both ends.
//
// With a certified JKR solver, a pair whose JKR force needs the reference's
// own Newton iteration (up to 20 steps) is not evaluated in this pass: it
// would hold its whole warp for those steps. It is appended to
// a deferred list (contact_eval returns true) and k_contact_deferred
// evaluates the deferred pairs densely; each pair writes the same result slots
// in either pass, so the outcome does not depend on the order.
// One contact result (force and torque on the row's particle, times its
// visit count) into its record: FP64 in the FP64 form; FP32 in the mixed form,
// whose pair forces are FP32 values (24 bytes a record instead of 48; the
// per-particle sums stay FP64). Pairs the mixed form evaluates in FP64 (the
// JKR fold band, decisions within FP32 rounding) are rounded once here.
// The FP32 form's results stay FP32 from the law to the record (a visit
// count times an FP32 value rounds the same in FP32 as in FP64).
template <typename R>
__device__ __forceinline__ void put_result(const StepParams& P, uint32_t rec, T3<R> f, T3<R> t, int visits) {
  if (visits != 1) {  // x * 1 = x: no multiply for the common single visit
    const R s = (R)visits;
    f = f * s;
    t = t * s;
  }
  if (P.prec == 1) {
    float2* o = reinterpret_cast<float2*>(P.cresf + 6 * (size_t)rec);
    o[0] = make_float2((float)f.x, (float)f.y);
    o[1] = make_float2((float)f.z, (float)t.x);
    o[2] = make_float2((float)t.y, (float)t.z);
  } else {
    double2* o = reinterpret_cast<double2*>(P.cres + 6 * (size_t)rec);
    o[0] = make_double2(f.x, f.y);
    o[1] = make_double2(f.z, t.x);
    o[2] = make_double2(t.y, t.z);
  }
}

template <bool PHYS, bool HIST, typename R>
__device__ __forceinline__ bool contact_eval(const StepParams& P, const Bank& B, uint32_t t, bool first_pass,
                                             bool& excess, uint32_t* tally) {
  const size_t plane = (size_t)P.n * P.cap;
  const bool adh = (P.nmodel == 3 || P.nmodel == 4);
  const uint32_t s = P.clist[t];
  const uint32_t k = s / (uint32_t)P.cap, c = s - k * (uint32_t)P.cap;
  const CRec r = P.crec[s];
  const uint32_t j = r.j, m = r.mv & 0xFFFFu;
  const int vij = (r.mv >> 16) & 0xFF, vji = crec_vji(r.mv);
  const float guess = (first_pass && (r.mv & CREC_NET)) ? P.jguess[t] : -1.0f;
  if (tally && (r.mv & CREC_NET)) tally[3] += 1;
  const D4 xi4 = B.xr[k], xj4 = B.xr[j];
  const V d = mic(P, xyz(xi4) - xyz(xj4));
  const double d2 = dot(d, d);
  const double rsum = xi4.w + xj4.w;
  const double cut = rsum + (adh ? rsum * 0.5 : 0.0);
  const bool in = d2 < cut * cut;
  const size_t hik = (size_t)k * P.cap + m;
  double* hk = HIST ? B.hist + hik : nullptr;
  T3<R> fc = t3(R(0), R(0), R(0)), tc = fc, nrm = fc;
  if (in) {
    const D4 vi4 = B.vm[k], wi4 = B.wc[k], vj4 = B.vm[j], wj4 = B.wc[j];
    const Law lw = law_of(P, B, (int)k);
    bool deferred = false;
    const bool can_defer = first_pass && P.jfb != nullptr;
    if (!pair_contact<R, PHYS, HIST>(P, lw, d, d2, rsum, xi4.w, xj4.w, vi4.w, vj4.w, xyz(vi4), xyz(vj4), xyz(wi4),
                                     xyz(wj4), hk, plane, fc, tc, nrm, excess, guess, tally,
                                     can_defer ? &deferred : nullptr, !first_pass)) {
      V fd, td, nd;
      pair_contact<double, PHYS, HIST>(P, lw, d, d2, rsum, xi4.w, xj4.w, vi4.w, vj4.w, xyz(vi4), xyz(vj4),
                                       xyz(wi4), xyz(wj4), hk, plane, fd, td, nd, excess, guess, nullptr, nullptr,
                                       !first_pass);
      fc = cvt<R>(fd);
      tc = cvt<R>(td);
      nrm = cvt<R>(nd);
    }
    if (deferred) return true;
    if (HIST && m < 64) atomicOr(B.hmask + k, 1ull << m);
  } else if (HIST) {
    hk[0] = 0.0;
    hk[plane] = 0.0;
    hk[2 * plane] = 0.0;
  }
  if (P.debug) P.dbgMult[hik] = (uint8_t)(in ? vij : 0);
  put_result(P, P.coff[k] + c, fc, tc, vij);
  if (vji > 0) {
    const uint32_t nj = P.ccnt[j];
    const CRec* rj = P.crec + (size_t)j * P.cap;
    for (uint32_t c2 = 0; c2 < nj; ++c2) {
      if (rj[c2].j != k) continue;
      const T3<R> f2 = -fc;
      const T3<R> t2 = cross(nrm * (R)xj4.w, f2);
      put_result(P, P.coff[j] + c2, f2, t2, vji);
      const size_t h2 = (size_t)j * P.cap + (rj[c2].mv & 0xFFFFu);
      if (HIST) {
        B.hist[h2] = -hk[0];
        B.hist[plane + h2] = -hk[plane];
        B.hist[2 * plane + h2] = -hk[2 * plane];
        const uint32_t m2 = rj[c2].mv & 0xFFFFu;
        if (m2 < 64) atomicOr(B.hmask + j, 1ull << m2);
      }
      if (P.debug) P.dbgMult[h2] = (uint8_t)(in ? vji : 0);
      break;
    }
  }
  return false;
}

// A wall candidate of the filter: the FP64 sphere-triangle contact
// (src/simulation.rs:464-523); its force and torque are kept for
// k_accumulate, which adds them after the pair contacts in mesh order.
__device__ __forceinline__ void wall_eval(const StepParams& P, const Bank& B, uint32_t w, bool& excess) {
  const uint2 e = P.warena[w];
  const int k = (int)e.x;
  const D4 xi = B.xr[k], vi = B.vm[k], wi = B.wc[k];
  V fc, tc;
  const bool ok = wall_contact(P, law_of(P, B, k), P.tri[e.y], xyz(xi), xyz(vi), xyz(wi), xi.w, vi.w, fc, tc, excess);
  if (ok) {
    double2* o = reinterpret_cast<double2*>(P.wres + 6 * (size_t)w);
    o[0] = make_double2(fc.x, fc.y);
    o[1] = make_double2(fc.z, tc.x);
    o[2] = make_double2(tc.y, tc.z);
  }
  P.wok[w] = ok ? 1 : 0;
}

// Pass 3: one thread per evaluating record, then one per wall candidate (the
// few wall contacts spread over the whole grid with the pairs).
template <bool PHYS, bool HIST, typename R>
__global__ void __launch_bounds__(256) k_contact_force(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  const uint32_t total = P.ctot[1];
  const uint32_t items = total + (P.ntri > 0 ? min(P.ctot[4], P.wcap) : 0u);
  bool excess = false;
  uint32_t tally[6] = {0u, 0u, 0u, 0u, 0u, 0u};
  const int lane = threadIdx.x & 31;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < items; t += gridDim.x * blockDim.x) {
    bool deferred = false;
    if (t < total) deferred = contact_eval<PHYS, HIST, R>(P, B, t, true, excess, tally);
    else wall_eval(P, B, t - total, excess);
    // append the deferred pairs with one atomic per warp
    const unsigned act = __activemask();
    const unsigned bal = __ballot_sync(act, deferred);
    if (bal) {
      const int leader = __ffs(bal) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(P.ctot + 3, (uint32_t)__popc(bal));
      base = __shfl_sync(act, base, leader);
      if (deferred) P.jfb[base + (uint32_t)__popc(bal & ((1u << lane) - 1u))] = t;
    }
  }
  if (excess) C->overlap_flag = 1;
  if (P.jkr_solver != 0 && P.nmodel == 3) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const uint32_t v = __reduce_add_sync(0xFFFFFFFFu, tally[q]);
      if ((threadIdx.x & 31) == 0 && v) atomicAdd(&C->jkr_count[q], (unsigned long long)v);
    }
  }
}

// The deferred pairs of k_contact_force, one thread each, with the
// reference's Newton iteration for their JKR force.
template <bool PHYS, bool HIST, typename R>
__global__ void __launch_bounds__(128) k_contact_deferred(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  const uint32_t total = P.ctot[3];
  bool excess = false;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
    contact_eval<PHYS, HIST, R>(P, B, P.jfb[i], false, excess, nullptr);
  if (excess) C->overlap_flag = 1;
}

// Pass 4: per particle, the contact results in list order, then the wall
// contacts in mesh order, then a = g + F/m and tau = T
// (src/simulation.rs:265-271, 464-536). The wall candidates were listed by
// the filter (FP32 pretests against the triangles of the particle's
// triangle-grid cell) and evaluated by the pair kernel, one thread each, so
// F and T are the same sums as one thread walking its triangles.
// k_accumulate takes the slots in the order P.aorder, set at each list
// rebuild, so that a warp's lanes run loops of similar length; no order
// changes a result.
constexpr uint32_t ACC_BINS = 128;
constexpr uint32_t ACC_TILE = 256;
constexpr uint32_t ACC_SORT_BINS = 32;  // record counts up to 31 (more share the last bin)

__device__ __forceinline__ bool tri_cell_nonempty(const StepParams& P, float4 xf) {
  uint32_t s, e;
  return tri_cell_range(P, xf, s, e) && e > s;
}

// Whether no triangle can come within reach of a particle at xf (its
// position at a list rebuild) before the next rebuild: until then it moves
// less than half the skin, which is less than a triangle-grid cell
// (wall_far_ok), so its cell stays among the 27 around the present one, and
// all of those list no triangle; nor can it wrap across a periodic face,
// which moves it to another part of the mesh.
__device__ bool wall_far(const StepParams& P, float4 xf) {
  const float p[3] = {xf.x, xf.y, xf.z};
  float q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (P.periodic[a]) {
      const float lo = (float)P.bmin[a], hi = (float)P.bmax[a];
      if (!(p[a] - lo > P.wall_far_gap && hi - p[a] > P.wall_far_gap)) return false;
    }
    q[a] = floorf((p[a] - P.tminf[a]) * P.tinvf);
    if (!(q[a] == q[a])) return false;  // NaN
    if (q[a] + 1.0f < 0.0f || q[a] - 1.0f >= (float)P.tdims[a]) return true;  // the 27 cells lie outside the grid
  }
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int cx = (int)q[0] + dx, cy = (int)q[1] + dy, cz = (int)q[2] + dz;
        if (cx < 0 || cy < 0 || cz < 0 || cx >= P.tdims[0] || cy >= P.tdims[1] || cz >= P.tdims[2]) continue;
        const uint32_t cell = (uint32_t)cx + (uint32_t)P.tdims[0] * ((uint32_t)cy + (uint32_t)P.tdims[1] * (uint32_t)cz);
        if (P.tstart[cell + 1] > P.tstart[cell]) return false;
      }
  return true;
}

// The visiting order of k_accumulate, at a list rebuild: within each tile of
// 256 slots a counting sort by (triangles listed in the triangle-grid cell,
// Verlet-list length), dead slots after the live ones. Reads the bank the
// rebuild fills.
__global__ void __launch_bounds__(ACC_TILE) k_accum_order(StepParams P) {
  {
    volatile const Ctrl* c = P.ctrl;
    if (c->rebuild == 0 || c->halt != 0) return;
  }
  const Bank B = P.bank[P.ctrl->bank ^ 1];
  __shared__ uint32_t bins[ACC_BINS];
  for (int base = blockIdx.x * ACC_TILE; base < P.n; base += gridDim.x * ACC_TILE) {
    const int k0 = base + threadIdx.x;
    // keys: 0..62 no triangles, 63 dead, 64..126 triangles, 127 past the end
    uint32_t key = ACC_BINS - 1;
    if (k0 < P.n) {
      const uint32_t fl = B.flags[k0];
      if (fl & PF_DEAD) {
        key = 63;
      } else {
        key = min(B.ncnt[k0], 62u);
        const float4 xf = B.xf[k0];
        if (P.ntri > 0 && tri_cell_nonempty(P, xf)) key += 64;
        const bool far = P.ntri > 0 && P.wall_far_ok && wall_far(P, xf);
        B.flags[k0] = far ? (fl | PF_WALLFAR) : (fl & ~PF_WALLFAR);
      }
    }
    for (uint32_t i = threadIdx.x; i < ACC_BINS; i += blockDim.x) bins[i] = 0;
    __syncthreads();
    const uint32_t rank = atomicAdd(&bins[key], 1u);
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive scan of the bins, four per lane
      const uint32_t l = threadIdx.x;
      const uint32_t c0 = bins[4 * l], c1 = bins[4 * l + 1], c2 = bins[4 * l + 2], c3 = bins[4 * l + 3];
      const uint32_t sum = c0 + c1 + c2 + c3;
      uint32_t incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= (uint32_t)o) incl += t;
      }
      const uint32_t ex = incl - sum;
      bins[4 * l] = ex;
      bins[4 * l + 1] = ex + c0;
      bins[4 * l + 2] = ex + c0 + c1;
      bins[4 * l + 3] = ex + c0 + c1 + c2;
    }
    __syncthreads();
    if (k0 < P.n) P.aorder[base + bins[key] + rank] = (uint32_t)k0;
    __syncthreads();
  }
}

int launch_accum_order(const StepParams& P, cudaStream_t s) {
  const uint64_t tiles = ((uint64_t)P.n + ACC_TILE - 1) / ACC_TILE;
  k_accum_order<<<(int)std::min<uint64_t>(std::max<uint64_t>(tiles, 1), (uint64_t)P.nsm * 64ull), ACC_TILE, 0, s>>>(P);
  return 1;
}

// Exclusive scan of one value per thread (blockDim.x a multiple of 32, at
// most 256); the block total goes to *total. Contains two __syncthreads.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* wsum, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < nw ? wsum[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= (uint32_t)o) wi += t;
    }
    if (lane < nw) wsum[lane] = wi - w;
    if (lane == nw - 1) *total = wi;
  }
  __syncthreads();
  return inc - v + wsum[warp];
}

// a = g + F (1/m) and tau = 0 + T for one particle, with the debug record and
// the non-finite check (on the integer pipe, as the +0 of 0 + T).
__device__ __forceinline__ void finish_particle(const StepParams& P, const Bank& B, Ctrl* C, int k, V F, V T) {
  if (P.debug) {
    P.dbgF[3 * (size_t)k] = F.x; P.dbgF[3 * (size_t)k + 1] = F.y; P.dbgF[3 * (size_t)k + 2] = F.z;
    P.dbgT[3 * (size_t)k] = T.x; P.dbgT[3 * (size_t)k + 1] = T.y; P.dbgT[3 * (size_t)k + 2] = T.z;
  }
  if (!(finite_bits(F.x) & finite_bits(F.y) & finite_bits(F.z) & finite_bits(T.x) & finite_bits(T.y) &
        finite_bits(T.z)))
    atomicOr(&C->status, (unsigned)ST_NAN);
  const V a = vmk(P.gravity[0], P.gravity[1], P.gravity[2]) + F * B.vres[k].w;  // F (1/m)
  B.acc[k] = D4{a.x, a.y, a.z, 0.0};
  B.tq[k] = D4{plus_zero(T.x), plus_zero(T.y), plus_zero(T.z), 0.0};
}

// Threads take the slots in the order aorder gives (tiles of 256 sorted by
// list length, particles in triangle cells last). The contact results are
// FP64 records (the FP64 form) or FP32 records (the mixed form, whose pair
// forces are FP32 values); either way the sums are FP64, in list order.
template <bool F32REC>
__global__ void __launch_bounds__(256) k_accumulate(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  // Each block takes a tile of blockDim.x slots (in aorder) and deals them
  // to its threads by their record and wall counts (a counting sort in shared
  // memory), so the lanes of a warp run sum loops of about the same length:
  // a partly filled FP64 warp instruction costs the pipe as much as a full one.
  __shared__ uint32_t bins[ACC_SORT_BINS];
  __shared__ int dealt[256];
  for (int base = blockIdx.x * blockDim.x; base < P.n; base += gridDim.x * blockDim.x) {
    const int i = base + (int)threadIdx.x;
    int k = -1;
    uint32_t key = 0;
    if (i < P.n) {
      k = (int)P.aorder[i];
      if (B.flags[k] & PF_DEAD) k = -1;
      else key = min(P.ccnt[k] + (P.ntri > 0 ? P.wcnt[k] : 0u), ACC_SORT_BINS - 1);
    }
    for (uint32_t b = threadIdx.x; b < ACC_SORT_BINS; b += blockDim.x) bins[b] = 0;
    __syncthreads();
    const uint32_t rank = atomicAdd(&bins[key], 1u);
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive scan of the bins, one per lane
      const uint32_t c0 = bins[threadIdx.x];
      uint32_t incl = c0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (threadIdx.x >= (uint32_t)o) incl += t;
      }
      bins[threadIdx.x] = incl - c0;
    }
    __syncthreads();
    dealt[bins[key] + rank] = k;
    __syncthreads();
    k = dealt[threadIdx.x];
    __syncthreads();
    if (k < 0) continue;
    V F = vmk(0.0, 0.0, 0.0), T = vmk(0.0, 0.0, 0.0);
    const uint32_t n = P.ccnt[k];
    if (F32REC) {
      // the mixed form's FP32 pair forces summed in FP32 (in list order, from
      // zero; the rounding adds at most (n - 1) 2^-24 of the sum of the
      // magnitudes), then widened exactly
      const float2* res = reinterpret_cast<const float2*>(P.cresf + 6 * (size_t)P.coff[k]);
      float fx = 0.0f, fy = 0.0f, fz = 0.0f, tx = 0.0f, ty = 0.0f, tz = 0.0f;
      for (uint32_t c = 0; c < n; ++c) {
        const float2 r0 = res[3 * c], r1 = res[3 * c + 1], r2 = res[3 * c + 2];
        fx = fx + r0.x; fy = fy + r0.y; fz = fz + r1.x;
        tx = tx + r1.y; ty = ty + r2.x; tz = tz + r2.y;
      }
      F = vmk(f2d_exact(fx), f2d_exact(fy), f2d_exact(fz));
      T = vmk(f2d_exact(tx), f2d_exact(ty), f2d_exact(tz));
    } else {
      const double2* res = reinterpret_cast<const double2*>(P.cres + 6 * (size_t)P.coff[k]);
      for (uint32_t c = 0; c < n; ++c) {
        const double2 r0 = res[3 * c], r1 = res[3 * c + 1], r2 = res[3 * c + 2];
        F = F + vmk(r0.x, r0.y, r1.x);
        T = T + vmk(r1.y, r2.x, r2.y);
      }
    }
    // the wall contacts (FP64 in both forms) after the pair contacts, in mesh order
    if (P.ntri > 0) {
      const uint32_t wn = P.wcnt[k], wo = P.woff[k];
      for (uint32_t c = 0; c < wn; ++c) {
        if (!P.wok[wo + c]) continue;
        const double2* r = reinterpret_cast<const double2*>(P.wres + 6 * (size_t)(wo + c));
        const double2 r0 = r[0], r1 = r[1], r2 = r[2];
        F = F + vmk(r0.x, r0.y, r1.x);
        T = T + vmk(r1.y, r2.x, r2.y);
      }
    }
    finish_particle(P, B, C, k, F, T);
  }
}

__global__ void k_clear_pending(StepParams P) {
  if (!P.ctrl->halt) P.ctrl->pending = 0;
}

// End of a step: count it and, inside the device step loop, decide whether
// the loop runs again. The loop also stops on a halt and after target + 4
// iterations whatever the counters say, so it always terminates.
__global__ void k_end_step(StepParams P, cudaGraphConditionalHandle loop, int in_loop) {
  Ctrl* C = P.ctrl;
  if (!C->halt) {
    C->steps_done += 1;
    C->pending = 1;
    if (C->overlap_flag) {
      C->overlap_steps += 1;
      C->status |= ST_OVERLAP;
      C->overlap_flag = 0;
    }
  }
  if (in_loop) {
    C->iters += 1;
    const bool again = !C->halt && C->steps_done < C->target && C->iters < C->target + 4;
    cudaGraphSetConditional(loop, again ? 1u : 0u);
  }
}

// Inside the device step loop: run the rebuild chain only when requested.
__global__ void k_rebuild_condition(StepParams P, cudaGraphConditionalHandle h) {
  const Ctrl* C = P.ctrl;
  cudaGraphSetConditional(h, (C->rebuild && !C->halt) ? 1u : 0u);
}

__global__ void k_kinetic(StepParams P, double* out) {
  const Bank B = P.bank[P.ctrl->bank];
  double e = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    if (B.flags[k] & PF_DEAD) continue;
    D4 v = B.vm[k], w = B.wc[k], x = B.xr[k];
    double I = 0.4 * v.w * x.w * x.w;
    e += 0.5 * v.w * (v.x * v.x + v.y * v.y + v.z * v.z) + 0.5 * I * (w.x * w.x + w.y * w.y + w.z * w.z);
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xFFFFFFFFu, e, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, e);
}

// Bed statistics of the live slots: out[0] kinetic energy (translational and
// rotational, I = 2/5 m r^2), out[1] the summed sphere volumes, *pairs the
// overlapping pairs counted from both ends over the Verlet lists (the exact
// FP64 test d^2 < (r_i + r_j)^2 on the minimum image; every such pair is in
// the lists, which hold all pairs within the cutoff plus the skin).
__global__ void k_bed_stats(StepParams P, double* out, unsigned long long* pairs) {
  const Bank B = P.bank[P.ctrl->bank];
  double e = 0.0, vol = 0.0;
  unsigned long long cnt = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    if (B.flags[k] & PF_DEAD) continue;
    const D4 v = B.vm[k], w = B.wc[k], x = B.xr[k];
    const double I = 0.4 * v.w * x.w * x.w;
    e += 0.5 * v.w * (v.x * v.x + v.y * v.y + v.z * v.z) + 0.5 * I * (w.x * w.x + w.y * w.y + w.z * w.z);
    vol += (4.0 / 3.0) * kPi * x.w * x.w * x.w;
    const uint32_t* row = B.nbr + (size_t)k * P.cap;
    const uint32_t c = B.ncnt[k];
    for (uint32_t m = 0; m < c; ++m) {
      const D4 y = B.xr[row[m]];
      const V d = mic(P, xyz(x) - xyz(y));
      const double rs = x.w + y.w;
      if (dot(d, d) < rs * rs) ++cnt;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_down_sync(0xFFFFFFFFu, e, o);
    vol += __shfl_down_sync(0xFFFFFFFFu, vol, o);
    cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], e);
    atomicAdd(&out[1], vol);
    atomicAdd(pairs, cnt);
  }
}

void launch_bed_stats(const StepParams& P, double* out, unsigned long long* pairs, cudaStream_t s) {
  cudaMemsetAsync(out, 0, 2 * sizeof(double), s);
  cudaMemsetAsync(pairs, 0, sizeof(unsigned long long), s);
  if (P.n == 0) return;
  k_bed_stats<<<grid_for(P.n, 256), 256, 0, s>>>(P, out, pairs);
}

int launch_first_half(const StepParams& P, cudaStream_t s) {
  if (P.n == 0) return 0;
  // the Kahan form holds 90 registers: blocks of 128 keep 20 warps resident
  // per multiprocessor where blocks of 256 keep 16
  if (P.prec == 1) k_first_half<false><<<grid_for(P.n, 256), 256, 0, s>>>(P);
  else k_first_half<true><<<grid_for(P.n, 128), 128, 0, s>>>(P);
  return 1;
}

int launch_second_half(const StepParams& P, cudaStream_t s) {
  if (P.n == 0) return 0;
  if (P.prec == 1) k_second_half<false><<<grid_for(P.n, 256), 256, 0, s>>>(P);
  else k_second_half<true><<<grid_for(P.n, 256), 256, 0, s>>>(P);
  k_clear_pending<<<1, 1, 0, s>>>(P);
  return 2;
}

int launch_rebuild_condition(const StepParams& P, cudaGraphConditionalHandle h, cudaStream_t s) {
  k_rebuild_condition<<<1, 1, 0, s>>>(P, h);
  return 1;
}

template <typename R>
static void launch_force_t(const StepParams& P, int g, cudaStream_t s) {
  const bool hist = P.mode == 1 && P.tmodel != 0;
  if (P.mode == 0) k_force<false, false, R><<<g, 128, 0, s>>>(P);
  else if (hist) k_force<true, true, R><<<g, 128, 0, s>>>(P);
  else k_force<true, false, R><<<g, 128, 0, s>>>(P);
}

// Grid for a grid-stride kernel of block `bs` over n items, at most `cap` blocks.
static int shaped_grid(uint64_t n, int bs, int cap) {
  uint64_t g = (n + (uint64_t)bs - 1) / (uint64_t)bs;
  if (g < 1) g = 1;
  if (g > (uint64_t)cap) g = (uint64_t)cap;
  return (int)g;
}

template <typename R>
static int launch_contact_path(const StepParams& P, cudaStream_t s) {
  const int bf = P.bs_filter > 0 ? P.bs_filter : 128, bc = P.bs_force > 0 ? P.bs_force : 128,
            ba = P.bs_accum > 0 ? P.bs_accum : 128, cap = P.grid_cap > 0 ? P.grid_cap : P.nsm * 64;
  const int g = shaped_grid((uint64_t)P.n, bf, cap);
  const bool hist = P.mode == 1 && P.tmodel != 0;
  cudaMemsetAsync(P.ctot, 0, sizeof(uint32_t) * CTOT_WORDS, s);
  if (P.mode == 0) k_contact_filter<false, false><<<g, bf, 0, s>>>(P);
  else if (hist) k_contact_filter<true, true><<<g, bf, 0, s>>>(P);
  else k_contact_filter<true, false><<<g, bf, 0, s>>>(P);
  const bool learn = P.jkr_solver == 1 && P.nmodel == 3 && P.mlp != nullptr;
  int launched = 3;
  if (learn) {
    k_jkr_mlp<<<P.nsm * 4, 128, 0, s>>>(P);
    ++launched;
  }
  const int gc = shaped_grid((uint64_t)P.n * 4, bc, cap);
  if (P.mode == 0) k_contact_force<false, false, R><<<gc, bc, 0, s>>>(P);
  else if (hist) k_contact_force<true, true, R><<<gc, bc, 0, s>>>(P);
  else k_contact_force<true, false, R><<<gc, bc, 0, s>>>(P);
  if (P.jfb != nullptr) {
    // the deferred pairs lie in the band next to the JKR fold, where only
    // FP64 resolves the contact radius: FP64 in the mixed form too
    if (P.mode == 0) k_contact_deferred<false, false, double><<<P.nsm * 8, 128, 0, s>>>(P);
    else if (hist) k_contact_deferred<true, true, double><<<P.nsm * 8, 128, 0, s>>>(P);
    else k_contact_deferred<true, false, double><<<P.nsm * 8, 128, 0, s>>>(P);
    ++launched;
  }
  if (P.prec == 1) k_accumulate<true><<<shaped_grid((uint64_t)P.n, ba, cap), ba, 0, s>>>(P);
  else k_accumulate<false><<<shaped_grid((uint64_t)P.n, ba, cap), ba, 0, s>>>(P);
  return launched;
}

int launch_force(const StepParams& P, cudaStream_t s) {
  if (P.n == 0) return 0;
  if (P.force_path == 0) return P.prec == 1 ? launch_contact_path<float>(P, s) : launch_contact_path<double>(P, s);
  const int g = grid_for(P.n, 128);
  if (P.prec == 1) launch_force_t<float>(P, g, s);
  else launch_force_t<double>(P, g, s);
  return 1;
}

int launch_end_step(const StepParams& P, cudaStream_t s) {
  k_end_step<<<1, 1, 0, s>>>(P, 0, 0);
  return 1;
}

int launch_end_step_loop(const StepParams& P, cudaGraphConditionalHandle loop, cudaStream_t s) {
  k_end_step<<<1, 1, 0, s>>>(P, loop, 1);
  return 1;
}

void launch_kinetic_energy(const StepParams& P, double* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(double), s);
  if (P.n == 0) return;
  k_kinetic<<<grid_for(P.n, 256), 256, 0, s>>>(P, out);
}

// ------------------------------------------------------- bulk state transfer
// The arrays of rp_read_state / rp_write_state are in id order; a slot's
// `tag` is its id (the particle's rank at the last upload), so slot_of[id]
// is a scatter of the tags. Used while no slot is dead (ids are then exactly
// 0..n-1). Copies only: no arithmetic touches the values.
__global__ void k_slot_of(StepParams P, uint32_t* slot_of, uint32_t* live) {
  const Bank B = P.bank[P.ctrl->bank];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    const uint32_t t = B.tag[k];
    slot_of[t] = (uint32_t)k;
    live[t] = (B.flags[k] & PF_DEAD) ? 0u : 1u;
  }
}

// With removed particles the ids are the live particles in upload order:
// id = the exclusive scan of the live flags at the upload position.
__global__ void k_compact_ids(int n, const uint32_t* slot_of, const uint32_t* live, const uint32_t* pos,
                              uint32_t* slot_of_id) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    if (live[t]) slot_of_id[pos[t]] = slot_of[t];
}

__global__ void k_state_gather(StepParams P, const uint32_t* slot_of, StateIO io, int m) {
  const Bank B = P.bank[P.ctrl->bank];
  const D4* src[8] = {B.xr, B.vm, B.wc, B.acc, B.tq, B.xres, B.vres, B.wres};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t k = slot_of[i];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (io.v[q]) {
        const D4 d = src[q][k];
        io.v[q][3 * (size_t)i] = d.x;
        io.v[q][3 * (size_t)i + 1] = d.y;
        io.v[q][3 * (size_t)i + 2] = d.z;
      }
    if (io.radius) io.radius[i] = B.xr[k].w;
    if (io.mass) io.mass[i] = B.vm[k].w;
    if (io.fixed) io.fixed[i] = (B.flags[k] & PF_FIXED) ? 1 : 0;
  }
}

// Whether the given radii, masses and fixed flags equal the current ones (the
// per-particle constants derived from them then stay valid).
__global__ void k_state_same(StepParams P, const uint32_t* slot_of, StateIO io, unsigned* differs, int m) {
  const Bank B = P.bank[P.ctrl->bank];
  bool d = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t k = slot_of[i];
    if (io.radius && __double_as_longlong(io.radius[i]) != __double_as_longlong(B.xr[k].w)) d = true;
    if (io.mass && __double_as_longlong(io.mass[i]) != __double_as_longlong(B.vm[k].w)) d = true;
    if (io.fixed && (io.fixed[i] != 0) != ((B.flags[k] & PF_FIXED) != 0)) d = true;
  }
  if (d) atomicOr(differs, 1u);
}

// Writes the given vector arrays into the slots (the .w fields, radius, mass,
// cell code, 1/m and 1/I, are kept) and refreshes the FP32 position mirror.
__global__ void k_state_scatter(StepParams P, const uint32_t* slot_of, StateIO io, int m) {
  const Bank B = P.bank[P.ctrl->bank];
  D4* dst[8] = {B.xr, B.vm, B.wc, B.acc, B.tq, B.xres, B.vres, B.wres};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t k = slot_of[i];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (io.v[q]) {
        D4 d = dst[q][k];
        d.x = io.v[q][3 * (size_t)i];
        d.y = io.v[q][3 * (size_t)i + 1];
        d.z = io.v[q][3 * (size_t)i + 2];
        dst[q][k] = d;
      }
    if (io.v[0]) {
      const D4 x = B.xr[k];
      B.xf[k] = make_float4((float)x.x, (float)x.y, (float)x.z, (float)x.w);
    }
  }
}

const uint32_t* launch_slot_of(const StepParams& P, const IdMap& M, int live, int n_ids, cudaStream_t s) {
  if (P.n == 0) return M.slot_of;
  // after a compaction some upload positions have no slot: their flags stay 0
  if (n_ids > P.n) cudaMemsetAsync(M.live, 0, sizeof(uint32_t) * (size_t)n_ids, s);
  k_slot_of<<<grid_for(P.n, 256), 256, 0, s>>>(P, M.slot_of, M.live);
  if (live == n_ids) return M.slot_of;  // nothing removed since the upload: the ids are the upload positions
  launch_exclusive_scan(nullptr, M.live, M.pos, (uint32_t)n_ids, M.part, nullptr, s);
  k_compact_ids<<<grid_for(n_ids, 256), 256, 0, s>>>(n_ids, M.slot_of, M.live, M.pos, M.slot_of_id);
  return M.slot_of_id;
}

void launch_state_gather(const StepParams& P, const uint32_t* slot_of, const StateIO& io, int m, cudaStream_t s) {
  if (m == 0) return;
  k_state_gather<<<grid_for(m, 256), 256, 0, s>>>(P, slot_of, io, m);
}

void launch_state_same(const StepParams& P, const uint32_t* slot_of, const StateIO& io, unsigned* differs, int m,
                       cudaStream_t s) {
  cudaMemsetAsync(differs, 0, sizeof(unsigned), s);
  if (m == 0) return;
  k_state_same<<<grid_for(m, 256), 256, 0, s>>>(P, slot_of, io, differs, m);
}

void launch_state_scatter(const StepParams& P, const uint32_t* slot_of, const StateIO& io, int m, cudaStream_t s) {
  if (m == 0) return;
  k_state_scatter<<<grid_for(m, 256), 256, 0, s>>>(P, slot_of, io, m);
}

}  // namespace rp
