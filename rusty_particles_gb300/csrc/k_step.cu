// Per-step kernels of the DEM step: boundary + first half of velocity Verlet,
// the pair/wall force gather fused with the second half, and the end-of-step
// bookkeeping.
//
// This translation unit is compiled with -fmad=false: every double operation
// rounds exactly as the oracle's (-ffp-contract=off), so positions after the
// first half, cutoff decisions, normals and relative velocities are
// bit-identical to the reference algorithm evaluated in FP64 from the same
// state. Force magnitudes differ only where a transcendental is evaluated
// differently (delta^1.5 as delta*sqrt(delta)), well inside 1e-9 relative.
#include <cfloat>

#include "rp_device.cuh"
#include "rp_launch.h"

namespace rp {

struct V {
  double x, y, z;
};
__device__ __forceinline__ V vmk(double x, double y, double z) { return V{x, y, z}; }
__device__ __forceinline__ V operator+(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator-(V a) { return V{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V operator*(V a, double s) { return V{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V operator*(double s, V a) { return V{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V operator/(V a, double s) { return V{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V cross(V a, V r) { return V{a.y * r.z - r.y * a.z, a.z * r.x - r.z * a.x, a.x * r.y - r.x * a.y}; }
__device__ __forceinline__ double len(V a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ V xyz(const D4& d) { return V{d.x, d.y, d.z}; }

constexpr double kPi = 3.14159265358979323846;

// ------------------------------------------------------------- force laws
// src/physics.rs:49-70
__device__ __forceinline__ double lsd_mag(double overlap, double vn, double kn, double gn) {
  return fmax(kn * overlap - gn * vn, 0.0);
}
// src/physics.rs:86-129 (delta^1.5 evaluated as delta*sqrt(delta))
__device__ __forceinline__ double hertz_mag(double overlap, double vn, double es, double rs, double ms, double beta_abs) {
  if (overlap <= 0.0) return 0.0;
  double kn = (4.0 / 3.0) * es * sqrt(rs);
  double fe = kn * (overlap * sqrt(overlap));
  double kt = 2.0 * es * sqrt(rs * overlap);
  double cn = 2.0 * sqrt(ms * kt) * beta_abs;
  double fd = -cn * vn;
  return fmax(fe + fd, 0.0);
}
__device__ __forceinline__ double hertz_elastic_mag(double overlap, double es, double rs) {
  double kn = (4.0 / 3.0) * es * sqrt(rs);
  return overlap > 0.0 ? kn * (overlap * sqrt(overlap)) : 0.0;
}
// src/physics.rs:132-219 (Newton on a^2/R* - sqrt(C a) - delta = 0)
__device__ __forceinline__ double jkr_mag(double overlap, double es, double rs, double gamma) {
  if (gamma <= 0.0) return hertz_elastic_mag(overlap, es, rs);
  const double eight_pi = 8.0 * kPi;
  double c_val = eight_pi * gamma / es;
  double sqrt_c = sqrt(c_val);
  double a = overlap > 0.0 ? sqrt(rs * overlap) : rs * 0.5;
  for (int it = 0; it < 20; ++it) {
    if (a <= 0.0) a = 1e-9;
    double ts = sqrt(c_val * a);
    double f_val = a * a / rs - ts - overlap;
    double df = 2.0 * a / rs - 0.5 * sqrt_c / sqrt(a);
    if (fabs(df) < 1e-9) break;
    double da = f_val / df;
    double max_step = a * 0.5;
    double step = da;
    if (step < -max_step) step = -max_step;
    if (step > max_step) step = max_step;
    a = a - step;
    if (fabs(step) < 1e-6 * rs) break;
  }
  double ts = sqrt(c_val * a);
  double f_val = a * a / rs - ts - overlap;
  if (fabs(f_val) > 1e-3 * rs) return 0.0;
  if (a <= 0.0) return 0.0;
  double a3 = a * a * a;
  double term1 = 4.0 * es * a3 / (3.0 * rs);
  double term2 = sqrt(eight_pi * gamma * es * a3);
  double fm = term1 - term2;
  double f_pull = (-2.0 / 3.0) * kPi * gamma * rs;
  if (fm < f_pull) return 0.0;
  return fm;
}
// src/physics.rs:234-325
__device__ __forceinline__ double sjkr_mag(double overlap, double vn, double es, double rs, double gamma) {
  if (gamma <= 0.0) return hertz_elastic_mag(overlap, es, rs);
  double f_pull = 1.5 * kPi * gamma * rs;
  double term = 3.0 * (kPi * kPi) * (gamma * gamma) * rs / (es * es);
  double delta_c = -sqrt(term);
  if (overlap < delta_c) return 0.0;
  double coh = vn > 0.0 ? 1.0 : 0.0;
  double fh = overlap > 0.0 ? (4.0 / 3.0) * es * sqrt(rs) * (overlap * sqrt(overlap)) : 0.0;
  return fh - coh * f_pull;
}

// Normal force vector for the configured model. `vn_src` is the relative
// velocity the model sees (the reference passes Vec3::ZERO to the
// hysteretic particle-particle law, src/simulation.rs:409-411).
__device__ __forceinline__ V normal_force(int model, double overlap, V n, V rv, double es, double rs, double ms,
                                          double beta_abs, double gamma, bool wall) {
  double m;
  switch (model) {
    case 1: m = hertz_mag(overlap, dot(rv, n), es, rs, ms, beta_abs); break;
    case 0: {
      double kn = es * rs;
      double gn = 0.5 * sqrt(ms * kn);
      m = lsd_mag(overlap, dot(rv, n), kn, gn);
    } break;
    case 2: {
      double kn = es * rs;
      double vn = wall ? dot(rv, n) : dot(vmk(0.0, 0.0, 0.0), n);
      m = lsd_mag(overlap, vn, kn, 0.0);
    } break;
    case 3: m = jkr_mag(overlap, es, rs, gamma); break;
    default: m = sjkr_mag(overlap, dot(rv, n), es, rs, gamma); break;
  }
  return m * n;
}

// src/physics.rs:385-397
__device__ __forceinline__ V coulomb_force(double fn, V rv, V n, double mu) {
  V vt = rv - dot(rv, n) * n;
  if (dot(vt, vt) < 1e-8) return vmk(0.0, 0.0, 0.0);
  double inv = 1.0 / len(vt);
  V dir = vt * inv;
  return (-mu * fn) * dir;
}
// src/physics.rs:400-434 with the spring `xi` in registers.
__device__ __forceinline__ V spring_coulomb(double fn, V rv, V n, V& xi, double kt, double mu, double dt) {
  V vt = rv - dot(rv, n) * n;
  xi = xi + vt * dt;
  V trial = (-kt) * xi;
  double tm = len(trial);
  double fc = mu * fn;
  if (tm > fc) {
    V dir = tm > 1e-6 ? trial / tm : vmk(0.0, 0.0, 0.0);
    V ft = fc * dir;
    xi = (-ft) / kt;
    return ft;
  }
  return trial;
}

// Second half of velocity Verlet for one particle (src/simulation.rs:541-561):
// Kahan-compensated v += a dt/2 and omega += (tau/I) dt/2, I = 0.4 m r^2.
__device__ __forceinline__ void second_half_kick(V& v, V& vres, V& w, V& wres, V a, V tau, double m, double r,
                                                 double dt) {
  V dv = (0.5 * a) * dt;
  V yv = dv - vres;
  V tv = v + yv;
  vres = (tv - v) - yv;
  v = tv;
  double inertia = 0.4 * m * r * r;
  V aa = tau / inertia;
  V dw = (0.5 * aa) * dt;
  V yw = dw - wres;
  V tw = w + yw;
  wres = (tw - w) - yw;
  w = tw;
}

// ------------------------------------------------------------- first half
// The force kernel only writes a and tau: neighbours read v and omega while
// it runs, so the second half kick of step n-1 is applied here, at the start
// of step n (FUSE), and by k_second_half at the end of a stepping call.
// Then src/simulation.rs:176-263: periodic wrap, out-of-bounds removal
// (marked dead here and compacted by the host later; removal changes no other
// particle's update), Kahan-compensated half kick + drift + angular half
// kick. Also records the reference-grid cell code and requests a list
// rebuild when a particle moved more than half the skin since the last build.
template <bool FUSE>
__global__ void __launch_bounds__(256) k_first_half(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  const double dt = P.dt;
  const bool anyp = P.periodic[0] | P.periodic[1] | P.periodic[2];
  const float half_skin = (float)(0.5 * P.skin);
  bool want_rebuild = false;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t fl = B.flags[k];
    if (fl & PF_DEAD) continue;
    D4 xr = B.xr[k], vm = B.vm[k], wc = B.wc[k];
    V x = xyz(xr), v = xyz(vm), w = xyz(wc);
    const bool moving = !(fl & PF_FIXED);
    V a = vmk(0.0, 0.0, 0.0), tau = a, vres = a, wres = a, xres = a;
    if (moving) {
      a = xyz(B.acc[k]);
      tau = xyz(B.tq[k]);
      vres = xyz(B.vres[k]);
      wres = xyz(B.wres[k]);
      xres = xyz(B.xres[k]);
      if (FUSE) second_half_kick(v, vres, w, wres, a, tau, vm.w, xr.w, dt);
    }
    if (anyp) {
      if (P.periodic[0]) { if (x.x < P.bmin[0]) x.x = x.x + P.bsize[0]; else if (x.x >= P.bmax[0]) x.x = x.x - P.bsize[0]; }
      if (P.periodic[1]) { if (x.y < P.bmin[1]) x.y = x.y + P.bsize[1]; else if (x.y >= P.bmax[1]) x.y = x.y - P.bsize[1]; }
      if (P.periodic[2]) { if (x.z < P.bmin[2]) x.z = x.z + P.bsize[2]; else if (x.z >= P.bmax[2]) x.z = x.z - P.bsize[2]; }
    }
    bool keep = (P.periodic[0] || (x.x >= P.bmin[0] - 1.0 && x.x <= P.bmax[0] + 1.0)) &&
                (P.periodic[1] || (x.y >= P.bmin[1] - 1.0)) &&
                (P.periodic[2] || (x.z >= P.bmin[2] - 1.0 && x.z <= P.bmax[2] + 1.0));
    if (!keep) {
      B.flags[k] = fl | PF_DEAD;
      const double nan = __longlong_as_double(0x7ff8000000000000ll);
      xr.x = nan; xr.y = nan; xr.z = nan;
      B.xr[k] = xr;
      atomicAdd(&C->removed, 1ull);
      continue;
    }
    if (moving) {
      V dv = (0.5 * a) * dt;
      V yv = dv - vres;
      V tv = v + yv;
      vres = (tv - v) - yv;
      v = tv;
      V dx = v * dt;
      V yx = dx - xres;
      V tx = x + yx;
      xres = (tx - x) - yx;
      x = tx;
      double inertia = 0.4 * vm.w * xr.w * xr.w;
      V aa = tau / inertia;
      V dw = (0.5 * aa) * dt;
      V yw = dw - wres;
      V tw = w + yw;
      wres = (tw - w) - yw;
      w = tw;
      B.vm[k] = D4{v.x, v.y, v.z, vm.w};
      B.vres[k] = D4{vres.x, vres.y, vres.z, 0.0};
      B.xres[k] = D4{xres.x, xres.y, xres.z, 0.0};
      B.wres[k] = D4{wres.x, wres.y, wres.z, 0.0};
      wc.x = w.x; wc.y = w.y; wc.z = w.z;
    }
    if (P.mode == 0) {
      int32_t c[3];
      ref_coords(P, x.x, x.y, x.z, c);
      wc.w = __longlong_as_double((long long)pack_code(c[0], c[1], c[2]));
    }
    B.wc[k] = wc;
    B.xr[k] = D4{x.x, x.y, x.z, xr.w};
    float4 r0 = B.xref[k];
    float ddx = (float)x.x - r0.x, ddy = (float)x.y - r0.y, ddz = (float)x.z - r0.z;
    if (P.periodic[0]) ddx -= (float)P.bsize[0] * rintf(ddx / (float)P.bsize[0]);
    if (P.periodic[1]) ddy -= (float)P.bsize[1] * rintf(ddy / (float)P.bsize[1]);
    if (P.periodic[2]) ddz -= (float)P.bsize[2] * rintf(ddz / (float)P.bsize[2]);
    float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
    if (!(d2 <= half_skin * half_skin)) want_rebuild = true;  // NaN (no build yet) also rebuilds
  }
  if (want_rebuild) C->rebuild = 1;
}

// Completes the last step of a stepping call (the pending second half).
__global__ void __launch_bounds__(256) k_second_half(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t fl = B.flags[k];
    if (fl & (PF_DEAD | PF_FIXED)) continue;
    D4 xr = B.xr[k], vm = B.vm[k], wc = B.wc[k];
    V v = xyz(vm), w = xyz(wc), vres = xyz(B.vres[k]), wres = xyz(B.wres[k]);
    second_half_kick(v, vres, w, wres, xyz(B.acc[k]), xyz(B.tq[k]), vm.w, xr.w, P.dt);
    B.vm[k] = D4{v.x, v.y, v.z, vm.w};
    B.wc[k] = D4{w.x, w.y, w.z, wc.w};
    B.vres[k] = D4{vres.x, vres.y, vres.z, 0.0};
    B.wres[k] = D4{wres.x, wres.y, wres.z, 0.0};
  }
}

// ------------------------------------------------- forces + second half
// One thread per slot gathers its Verlet list: the exact FP64 cutoff test
// of src/simulation.rs:327-357, the reference's visit count in parity mode,
// the pair laws of src/simulation.rs:372-460, the wall triangles of
// src/simulation.rs:464-523 from the triangle grid, then a += F/m, tau += T
// and the second Kahan half kick (src/simulation.rs:532-561).
template <bool PHYS, bool HIST>
__global__ void __launch_bounds__(128) k_force(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  const Bank B = P.bank[C->bank];
  const double dt = P.dt;
  const bool adh = (P.nmodel == 3 || P.nmodel == 4);
  const double beta_abs = P.beta_abs;
  const size_t plane = (size_t)P.n * P.cap;
  bool excess = false;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    const uint32_t fl = B.flags[k];
    if (fl & PF_DEAD) continue;
    const D4 xi4 = B.xr[k], vi4 = B.vm[k], wi4 = B.wc[k];
    const V xi = xyz(xi4), vi = xyz(vi4), wi = xyz(wi4);
    const double ri = xi4.w, mi = vi4.w;
    const unsigned long long ci = (unsigned long long)__double_as_longlong(wi4.w);
    V F = vmk(0.0, 0.0, 0.0), T = vmk(0.0, 0.0, 0.0);
    const uint32_t cnt = B.ncnt[k];
    const uint32_t* row = B.nbr + (size_t)k * P.cap;
    for (uint32_t m = 0; m < cnt; ++m) {
      const uint32_t j = row[m];
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
      if (d2 < cut * cut) {
        const D4 wj4 = B.wc[j];
        if (!PHYS) visits = ref_visits(P, ci, (unsigned long long)__double_as_longlong(wj4.w));
        else visits = 1;
        if (visits > 0) {
          const D4 vj4 = B.vm[j];
          const double dist = sqrt(d2);
          const double overlap = rsum - dist;
          if (overlap > 0.2 * fmin(ri, rj)) excess = true;
          const V n = dist > 1e-6 ? d / dist : vmk(0.0, 1.0, 0.0);
          const V ra = (-n) * ri;
          const V rb = n * rj;
          const V va = vi + cross(wi, ra);
          const V vb = xyz(vj4) + cross(xyz(wj4), rb);
          const V rv = va - vb;
          const double rs = (ri * rj) / (ri + rj);
          const double ms = (mi * vj4.w) / (mi + vj4.w);
          const V fnv = normal_force(P.nmodel, overlap, n, rv, P.es_pp, rs, ms, beta_abs, P.gamma_pp, false);
          const double fnm = len(fnv);
          V ft;
          if (P.tmodel == 0) {
            ft = coulomb_force(fnm, rv, n, P.pm.mu);
          } else if (!PHYS) {
            // G* = 0 (src/material.rs:39-50): the spring force is +-0, or NaN
            // when Mindlin takes sqrt of a negative overlap.
            double kt = P.tmodel == 2 ? 8.0 * P.gs_pp * sqrt(rs * overlap) : P.gs_pp * rs;
            ft = (kt != kt) ? vmk(kt, kt, kt) : vmk(0.0, 0.0, 0.0);
          } else {
            V xi_s = vmk(0.0, 0.0, 0.0);
            const size_t hi = (size_t)k * P.cap + m;
            if (overlap > 0.0) {
              double kt = P.tmodel == 2 ? 8.0 * P.gs_pp * sqrt(rs * overlap) : P.gs_pp * rs;
              if (HIST) xi_s = vmk(B.hist[hi], B.hist[plane + hi], B.hist[2 * plane + hi]);
              xi_s = xi_s - dot(xi_s, n) * n;
              ft = spring_coulomb(fnm, rv, n, xi_s, kt, P.pm.mu, dt);
            } else {
              ft = vmk(0.0, 0.0, 0.0);
            }
            if (HIST) {
              B.hist[hi] = xi_s.x;
              B.hist[plane + hi] = xi_s.y;
              B.hist[2 * plane + hi] = xi_s.z;
            }
          }
          const V fc = fnv + ft;
          const V tc = cross(ra, fc);
          for (int t = 0; t < visits; ++t) {
            F = F + fc;
            T = T + tc;
          }
        }
      }
      if (PHYS && HIST && visits == 0) {
        const size_t hi = (size_t)k * P.cap + m;
        B.hist[hi] = 0.0;
        B.hist[plane + hi] = 0.0;
        B.hist[2 * plane + hi] = 0.0;
      }
      if (P.debug) P.dbgMult[(size_t)k * P.cap + m] = (uint8_t)visits;
    }
    // walls: triangles of the particle's triangle-grid cell, in mesh order
    if (P.ntri > 0) {
      const double q0 = floor((xi.x - P.tmin[0]) / P.tcell);
      const double q1 = floor((xi.y - P.tmin[1]) / P.tcell);
      const double q2 = floor((xi.z - P.tmin[2]) / P.tcell);
      if (q0 >= 0.0 && q1 >= 0.0 && q2 >= 0.0 && q0 < (double)P.tdims[0] && q1 < (double)P.tdims[1] &&
          q2 < (double)P.tdims[2]) {
        const uint32_t cell = (uint32_t)q0 + (uint32_t)P.tdims[0] * ((uint32_t)q1 + (uint32_t)P.tdims[1] * (uint32_t)q2);
        const uint32_t s = P.tstart[cell], e = P.tstart[cell + 1];
        for (uint32_t t = s; t < e; ++t) {
          const TriRec& tr = P.tri[P.titems[t]];
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
          if (!(dsq < ri * ri)) continue;
          const double dist = sqrt(dsq);
          const double pen = ri - dist;
          const V n = dist > 1e-6 ? dv / dist : vmk(tr.n[0], tr.n[1], tr.n[2]);
          if (pen > 0.2 * ri) excess = true;
          const V ra = (-n) * ri;
          const V rv = vi + cross(wi, ra);
          const V fnv = normal_force(P.nmodel, pen, n, rv, P.es_pw, ri, mi, beta_abs, P.gamma_pw, true);
          const V fc = fnv + coulomb_force(len(fnv), rv, n, P.pm.mu);
          F = F + fc;
          T = T + cross(ra, fc);
        }
      }
    }
    if (P.debug) {
      P.dbgF[3 * (size_t)k] = F.x; P.dbgF[3 * (size_t)k + 1] = F.y; P.dbgF[3 * (size_t)k + 2] = F.z;
      P.dbgT[3 * (size_t)k] = T.x; P.dbgT[3 * (size_t)k + 1] = T.y; P.dbgT[3 * (size_t)k + 2] = T.z;
    }
    if (!isfinite(F.x + F.y + F.z + T.x + T.y + T.z)) atomicOr(&C->status, (unsigned)ST_NAN);
    // apply (src/simulation.rs:532-536); the second half kick of this step
    // runs in the next k_first_half or in k_second_half
    const V a = vmk(P.gravity[0], P.gravity[1], P.gravity[2]) + F / mi;
    const V tau = vmk(0.0, 0.0, 0.0) + T;
    B.acc[k] = D4{a.x, a.y, a.z, 0.0};
    B.tq[k] = D4{tau.x, tau.y, tau.z, 0.0};
  }
  if (excess) C->overlap_flag = 1;
}

__global__ void k_end_step(StepParams P) {
  Ctrl* C = P.ctrl;
  if (C->halt) return;
  C->steps_done += 1;
  if (C->overlap_flag) {
    C->overlap_steps += 1;
    C->status |= ST_OVERLAP;
    C->overlap_flag = 0;
  }
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

int launch_first_half(const StepParams& P, bool fuse_second_half, cudaStream_t s) {
  if (P.n == 0) return 0;
  if (fuse_second_half) k_first_half<true><<<grid_for(P.n, 256), 256, 0, s>>>(P);
  else k_first_half<false><<<grid_for(P.n, 256), 256, 0, s>>>(P);
  return 1;
}

int launch_second_half(const StepParams& P, cudaStream_t s) {
  if (P.n == 0) return 0;
  k_second_half<<<grid_for(P.n, 256), 256, 0, s>>>(P);
  return 1;
}

int launch_force(const StepParams& P, cudaStream_t s) {
  if (P.n == 0) return 0;
  const int g = grid_for(P.n, 128);
  const bool hist = P.mode == 1 && P.tmodel != 0;
  if (P.mode == 0) k_force<false, false><<<g, 128, 0, s>>>(P);
  else if (hist) k_force<true, true><<<g, 128, 0, s>>>(P);
  else k_force<true, false><<<g, 128, 0, s>>>(P);
  return 1;
}

int launch_end_step(const StepParams& P, cudaStream_t s) {
  k_end_step<<<1, 1, 0, s>>>(P);
  return 1;
}

void launch_kinetic_energy(const StepParams& P, double* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(double), s);
  if (P.n == 0) return;
  k_kinetic<<<grid_for(P.n, 256), 256, 0, s>>>(P, out);
}

}  // namespace rp
