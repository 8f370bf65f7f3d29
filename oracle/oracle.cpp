// CPU oracle for the rusty_particles DEM time step.
//
// TEST INFRASTRUCTURE ONLY. This file is a plain C++ restatement of the
// reference's CPU step (`Simulation::step_cpu`, src/simulation.rs:173-562) and
// of the modules it calls. It exists to check the CUDA product path and to
// time the reference's CPU algorithm as a baseline. The product library
// (rusty_particles_gb300) never links, loads or calls it.
//
// Arithmetic follows the reference operation by operation (glam `Vec3`
// semantics with the `scalar-math` feature, Rust operator precedence, Rust
// `f32::max`/`clamp` NaN behaviour), templated on float (the reference's own
// precision) and double (the FP64 oracle). Build with -ffp-contract=off so no
// fused multiply-add changes the rounding on either x86-64 or aarch64.
//
// Two interaction modes:
//   * parity   — the reference exactly: candidate pairs from the reference's
//                uniform grid (src/grid.rs:12-87, cell size 1.0 by default,
//                dims = ceil(size/h)+1, one periodic wrap of cell coords, 27
//                cells in z,y,x order, a cell listed twice is visited twice),
//                effective shear modulus 0 (src/material.rs:39-50), contact
//                history in a map keyed by (min,max) index and updated from
//                both sides (src/simulation.rs:397-399).
//   * physical — all minimum-image pairs within the cutoff, each visited
//                once; Mindlin G* from 1/G* = (2-nu1)/G1 + (2-nu2)/G2;
//                tangential history per directed pair keyed by a stable
//                particle tag, projected onto the contact plane each step and
//                erased when the pair leaves contact.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

template <typename T>
struct V3 {
  T x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(T a, T b, T c) : x(a), y(b), z(c) {}
  V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
  V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
  V3 operator-() const { return V3(-x, -y, -z); }
  V3 operator*(T s) const { return V3(x * s, y * s, z * s); }
  V3 operator/(T s) const { return V3(x / s, y / s, z / s); }
  V3& operator+=(const V3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
  // glam: dot = x*x' + y*y' + z*z' evaluated left to right.
  T dot(const V3& o) const { return x * o.x + y * o.y + z * o.z; }
  T length_squared() const { return dot(*this); }
  T length() const { return std::sqrt(dot(*this)); }
  V3 cross(const V3& r) const {
    return V3(y * r.z - r.y * z, z * r.x - r.z * x, x * r.y - r.x * y);
  }
  // glam normalize: self * (1 / length)
  V3 normalize() const { T inv = T(1) / length(); return *this * inv; }
};
template <typename T> inline V3<T> operator*(T s, const V3<T>& v) { return V3<T>(s * v.x, s * v.y, s * v.z); }

// Rust f32::max: IEEE maxNum, a NaN operand yields the other operand.
template <typename T> inline T rmax(T a, T b) { return std::fmax(a, b); }
// Rust f32::clamp(min, max) for min <= max: NaN passes through.
template <typename T> inline T rclamp(T v, T lo, T hi) {
  T r = v;
  if (r < lo) r = lo;
  if (r > hi) r = hi;
  return r;
}
// Rust `as i32` from a float: saturating, NaN -> 0.
template <typename T> inline int32_t sat_i32(T f) {
  if (std::isnan(f)) return 0;
  if (f <= T(-2147483648.0)) return INT32_MIN;
  if (f >= T(2147483647.0)) return INT32_MAX;
  return (int32_t)f;
}
template <typename T> inline T pi() { return T(3.14159265358979323846); }

enum NormalModel { N_LINEAR = 0, N_HERTZ = 1, N_HYSTERETIC = 2, N_JKR = 3, N_SJKR = 4 };
enum TangentialModel { T_COULOMB = 0, T_LINEAR_SPRING = 1, T_MINDLIN = 2 };
enum Mode { MODE_PARITY = 0, MODE_PHYSICAL = 1 };

template <typename T>
struct Material {  // src/material.rs:2-21
  T E, nu, rho, mu, e, gamma;
};

// src/material.rs:25-54
template <typename T> inline T effective_radius(T r1, T r2) { return (r1 * r2) / (r1 + r2); }
template <typename T> inline T effective_mass(T m1, T m2) { return (m1 * m2) / (m1 + m2); }
template <typename T> inline T effective_youngs(T e1, T nu1, T e2, T nu2) {
  T inv = (T(1) - nu1 * nu1) / e1 + (T(1) - nu2 * nu2) / e2;
  return T(1) / inv;
}
template <typename T> inline T shear_modulus(T e, T nu) { return e / (T(2) * (T(1) + nu)); }
// Physical-mode Mindlin combination: 1/G* = (2-nu1)/G1 + (2-nu2)/G2.
template <typename T> inline T physical_shear(T e1, T nu1, T e2, T nu2) {
  T g1 = shear_modulus(e1, nu1), g2 = shear_modulus(e2, nu2);
  return T(1) / ((T(2) - nu1) / g1 + (T(2) - nu2) / g2);
}

template <typename T>
struct Particle {  // src/particle.rs:4-37
  V3<T> x, v, a;
  T r, m;
  bool fixed;
  V3<T> xres, vres;
  V3<T> w, tau, wres;
  uint64_t tag;  // stable identity (physical-mode history key); not in the reference
};

template <typename T>
struct Contact {  // src/contact.rs:4-17
  V3<T> xi;
  T nfh = 0;
  uint64_t age = 0;
};

// ---------------------------------------------------------------- force laws
// Each law also adds the magnitudes of its additive terms to tl_terms: the
// scale at which a different rounding of the same formula can change the
// result (a difference of two nearly equal terms has no relative precision of
// its own). Tests use it to normalise per-particle force errors.
thread_local double tl_terms = 0.0;
// src/physics.rs:49-70
template <typename T>
V3<T> linear_spring_dashpot(T overlap, V3<T> n, V3<T> rv, T kn, T gn) {
  T vn = rv.dot(n);
  T f = kn * overlap - gn * vn;
  tl_terms += std::fabs((double)(kn * overlap)) + std::fabs((double)(gn * vn));
  f = rmax(f, T(0));
  return f * n;
}
// src/physics.rs:86-129
template <typename T>
V3<T> hertzian(T overlap, V3<T> n, V3<T> rv, T es, T rs, T ms, T e) {
  if (overlap <= T(0)) return V3<T>();
  T kn = T(4.0 / 3.0) * es * std::sqrt(rs);
  T fe = kn * std::pow(overlap, T(1.5));
  T ln_e = std::log(e);
  T beta = ln_e / std::sqrt(ln_e * ln_e + pi<T>() * pi<T>());
  T kt = T(2) * es * std::sqrt(rs * overlap);
  T cn = T(2) * std::sqrt(ms * kt) * std::fabs(beta);
  T vn = rv.dot(n);
  T fd = -cn * vn;
  tl_terms += std::fabs((double)fe) + std::fabs((double)fd);
  T tot = rmax(fe + fd, T(0));
  return tot * n;
}
// Hertz elastic fallback used by JKR/sJKR when gamma <= 0 (src/physics.rs:157-163, 243-248)
template <typename T>
V3<T> hertz_elastic(T overlap, V3<T> n, T es, T rs) {
  T kn = T(4.0 / 3.0) * es * std::sqrt(rs);
  T f = overlap > T(0) ? kn * std::pow(overlap, T(1.5)) : T(0);
  tl_terms += std::fabs((double)f);
  return f * n;
}
// The Newton iteration for the JKR contact radius, src/physics.rs:164-191;
// `iters` receives the number of loop bodies run.
template <typename T>
T jkr_radius(T overlap, T es, T rs, T gamma, int* iters) {
  const T eight_pi = T(8) * pi<T>();
  T c_val = eight_pi * gamma / es;
  T sqrt_c = std::sqrt(c_val);
  T a = overlap > T(0) ? std::sqrt(rs * overlap) : rs * T(0.5);
  int it = 0;
  while (it < 20) {
    ++it;
    if (a <= T(0)) a = T(1e-9);
    T ts = std::sqrt(c_val * a);
    T f_val = a * a / rs - ts - overlap;
    T df = T(2) * a / rs - T(0.5) * sqrt_c / std::sqrt(a);
    if (std::fabs(df) < T(1e-9)) break;
    T da = f_val / df;
    T max_step = a * T(0.5);
    T step = rclamp(da, -max_step, max_step);
    a = a - step;
    if (std::fabs(step) < T(1e-6) * rs) break;
  }
  if (iters) *iters = it;
  return a;
}
// src/physics.rs:132-219
template <typename T>
V3<T> jkr(T overlap, V3<T> n, T es, T rs, T gamma) {
  if (gamma <= T(0)) return hertz_elastic(overlap, n, es, rs);
  const T eight_pi = T(8) * pi<T>();
  T c_val = eight_pi * gamma / es;
  T a = jkr_radius(overlap, es, rs, gamma, (int*)nullptr);
  T ts = std::sqrt(c_val * a);
  T f_val = a * a / rs - ts - overlap;
  if (std::fabs(f_val) > T(1e-3) * rs) return V3<T>();
  if (a <= T(0)) return V3<T>();
  T a3 = a * a * a;
  T term1 = T(4) * es * a3 / (T(3) * rs);
  T term2 = std::sqrt(eight_pi * gamma * es * a3);
  T fm = term1 - term2;
  T f_pull = T(-2.0 / 3.0) * pi<T>() * gamma * rs;
  if (fm < f_pull) return V3<T>();
  tl_terms += std::fabs((double)term1) + std::fabs((double)term2);
  return fm * n;
}
// src/physics.rs:234-325
template <typename T>
V3<T> sjkr(T overlap, V3<T> n, V3<T> rv, T es, T rs, T gamma) {
  if (gamma <= T(0)) return hertz_elastic(overlap, n, es, rs);
  T f_pull = T(1.5) * pi<T>() * gamma * rs;
  T term = T(3) * (pi<T>() * pi<T>()) * (gamma * gamma) * rs / (es * es);
  T delta_c = -std::sqrt(term);
  if (overlap < delta_c) return V3<T>();
  T vn = rv.dot(n);
  T coh = vn > T(0) ? T(1) : T(0);
  T fh = overlap > T(0) ? T(4.0 / 3.0) * es * std::sqrt(rs) * std::pow(overlap, T(1.5)) : T(0);
  T tot = fh - coh * f_pull;
  tl_terms += std::fabs((double)fh) + std::fabs((double)(coh * f_pull));
  return tot * n;
}
// src/physics.rs:385-397
template <typename T>
V3<T> coulomb(T fn, V3<T> rv, V3<T> n, T mu) {
  V3<T> vt = rv - rv.dot(n) * n;
  if (vt.length_squared() < T(1e-8)) return V3<T>();
  V3<T> dir = vt.normalize();
  tl_terms += std::fabs((double)(mu * fn));
  return (-mu * fn) * dir;
}
// src/physics.rs:400-434 (xi is the stored tangential displacement)
template <typename T>
V3<T> linear_spring_coulomb(T fn, V3<T> rv, V3<T> n, V3<T>& xi, T kt, T mu, T dt) {
  V3<T> vt = rv - rv.dot(n) * n;
  xi += vt * dt;
  V3<T> trial = (-kt) * xi;
  T tm = trial.length();
  T fc = mu * fn;
  if (tm > fc) {
    V3<T> dir = tm > T(1e-6) ? trial / tm : V3<T>();
    V3<T> ft = fc * dir;
    xi = (-ft) / kt;
    tl_terms += (double)ft.length();
    return ft;
  }
  tl_terms += (double)trial.length();
  return trial;
}

// ------------------------------------------------------------ mesh triangles
template <typename T>
struct Triangle {  // src/mesh.rs:5-16
  V3<T> v0, v1, v2, n;
  int motion = -1;  // extension: index of a rigid surface velocity (-1: static, the reference's walls)
};
// Extension: the surface velocity V + W x (p - C) of a moving wall.
struct WallMotion {
  double c[3], w[3], v[3];
};
// src/mesh.rs:45-117 (region tests as in the reference, including its
// swapped (-e).clamp(0, c) assignment to s in the t<0 / a+d<=b+e branch)
template <typename T>
V3<T> closest_point(const Triangle<T>& tr, V3<T> p) {
  V3<T> e0 = tr.v1 - tr.v0, e1 = tr.v2 - tr.v0, v0 = tr.v0 - p;
  T a = e0.dot(e0), b = e0.dot(e1), c = e1.dot(e1), d = e0.dot(v0), e = e1.dot(v0);
  T det = a * c - b * b;
  T s = b * e - c * d;
  T t = b * d - a * e;
  T sc = s, tc = t;
  if (s + t < det) {
    if (s < T(0)) {
      if (t < T(0)) {
        if (d < T(0)) { sc = rclamp(-d, T(0), a); tc = T(0); }
        else { sc = T(0); tc = rclamp(-e, T(0), c); }
      } else { sc = T(0); tc = rclamp(-e, T(0), c); }
    } else if (t < T(0)) {
      sc = rclamp(-d, T(0), a); tc = T(0);
    } else {
      T inv = T(1) / det;
      sc = sc * inv; tc = tc * inv;
    }
  } else {
    if (s < T(0)) {
      T tmp0 = b + d, tmp1 = c + e;
      if (tmp1 > tmp0) {
        T numer = tmp1 - tmp0, denom = a - T(2) * b + c;
        sc = rclamp(numer / denom, T(0), T(1)); tc = T(1) - sc;
      } else { tc = rclamp(-e, T(0), c); sc = T(0); }
    } else if (t < T(0)) {
      if (a + d > b + e) {
        T numer = c + e - b - d, denom = a - T(2) * b + c;
        sc = rclamp(numer / denom, T(0), T(1)); tc = T(1) - sc;
      } else { sc = rclamp(-e, T(0), c); tc = T(0); }
    } else {
      T numer = c + e - b - d, denom = a - T(2) * b + c;
      sc = rclamp(numer / denom, T(0), T(1)); tc = T(1) - sc;
    }
  }
  return tr.v0 + sc * e0 + tc * e1;
}
// src/mesh.rs:20-43
template <typename T>
bool intersect_sphere(const Triangle<T>& tr, V3<T> c, T r, T& pen, V3<T>& n, V3<T>* cp_out = nullptr) {
  V3<T> cp = closest_point(tr, c);
  if (cp_out) *cp_out = cp;
  V3<T> dv = c - cp;
  T d2 = dv.length_squared();
  if (d2 < r * r) {
    T d = std::sqrt(d2);
    pen = r - d;
    n = d > T(1e-6) ? dv / d : tr.n;
    return true;
  }
  return false;
}

// -------------------------------------------------------------------- engine
struct Base {
  virtual ~Base() {}
};

template <typename T>
struct Sim : Base {
  T dt;
  V3<T> bmin, bmax;
  bool periodic[3] = {false, false, false};
  std::vector<Particle<T>> ps;
  std::vector<Triangle<T>> tris;
  std::vector<WallMotion> motions;
  Material<T> pm{T(1e7), T(0.3), T(2500), T(0.5), T(0.5), T(0)};   // src/simulation.rs:69
  Material<T> wm{T(1e9), T(0.3), T(7800), T(0.5), T(0.5), T(0)};   // src/simulation.rs:70
  int nmodel = N_HERTZ, tmodel = T_MINDLIN;                         // src/simulation.rs:84-85
  int mode = MODE_PARITY;
  T cell = T(1.0);                                                  // src/simulation.rs:66
  V3<T> gravity{T(0), T(-9.81), T(0)};                             // src/simulation.rs:267
  uint64_t next_tag = 0;
  uint64_t steps_done = 0;
  uint64_t overlap_warnings = 0;
  int warn_stderr = 0;

  // reference grid (CSR form of `cells: Vec<Vec<usize>>`, insertion order kept)
  int gd[3] = {0, 0, 0};
  std::vector<uint32_t> cell_start, cell_items;
  std::vector<int64_t> cell_of;  // per particle, -1 if not inserted

  // parity-mode contact map (DashMap<(usize,usize),Contact>), sharded locks
  static const int NSHARD = 64;
  std::unordered_map<uint64_t, Contact<T>> cmap[NSHARD];
  std::mutex cmut[NSHARD];
  bool keep_contact_map = true;

  // physical-mode per-particle history: sorted (tag_j, xi)
  struct Hist { uint64_t tag; V3<T> xi; };
  std::vector<std::vector<Hist>> hist;

  // Optional exact cull of the wall loop (a benchmark-side variant, off by
  // default): a uniform grid over the triangles, each listed in every cell
  // that its box grown by the largest radius overlaps. A sphere can only touch
  // a triangle when its centre lies in that grown box, so the triangles of the
  // centre's cell, in mesh order, give the same contacts in the same order as
  // the reference's every-triangle loop (src/simulation.rs:465-466).
  bool wall_cull = false;
  size_t cull_T = 0;
  T cull_rmax = T(-1), cull_h = T(1);
  V3<T> cull_lo;
  int cull_d[3] = {0, 0, 0};
  std::vector<uint32_t> cull_start, cull_items;

  // last-step diagnostics
  std::vector<V3<T>> lastF, lastT;
  std::vector<double> lastFS, lastTS;  // sums of |f_contact| and |r x f| per particle (summation-order scale)
  std::vector<uint64_t> pair_i, pair_j;  // pairs within cutoff, one entry per visit (i-side)
  bool record_pairs = false;
  std::mutex pair_mut;

  Sim(T dt_, V3<T> mn, V3<T> mx) : dt(dt_), bmin(mn), bmax(mx) {}

  void add_particle(V3<T> x, T r, T m, bool fixed) {
    Particle<T> p;
    p.x = x; p.r = r; p.m = m; p.fixed = fixed; p.tag = next_tag++;
    ps.push_back(p);
    hist.emplace_back();
  }

  int grid_dims() {
    V3<T> size = (bmax - bmin) / cell;
    int64_t d[3] = {(int64_t)sat_i32(std::ceil(size.x)) + 1, (int64_t)sat_i32(std::ceil(size.y)) + 1,
                    (int64_t)sat_i32(std::ceil(size.z)) + 1};
    for (int k = 0; k < 3; ++k) if (d[k] <= 0 || d[k] > (1 << 24)) return -1;
    if (d[0] * d[1] * d[2] > (int64_t)1 << 31) return -1;
    gd[0] = (int)d[0]; gd[1] = (int)d[1]; gd[2] = (int)d[2];
    return 0;
  }
  // src/grid.rs:30-40; coords saturate like Rust `as`.
  void cell_coords(V3<T> x, int32_t c[3]) const {
    V3<T> rel = x - bmin;
    V3<T> q = rel / cell;
    c[0] = sat_i32(std::floor(q.x)); c[1] = sat_i32(std::floor(q.y)); c[2] = sat_i32(std::floor(q.z));
  }
  int64_t cell_index(V3<T> x) const {
    int32_t c[3]; cell_coords(x, c);
    if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= gd[0] || c[1] >= gd[1] || c[2] >= gd[2]) return -1;
    return (int64_t)c[0] + (int64_t)c[1] * gd[0] + (int64_t)c[2] * gd[0] * gd[1];
  }
  // src/grid.rs:24-46 + src/simulation.rs:273-276 (serial insert in index order)
  void build_grid() {
    size_t nc = (size_t)gd[0] * gd[1] * gd[2];
    size_t n = ps.size();
    cell_of.assign(n, -1);
    cell_start.assign(nc + 1, 0);
    for (size_t i = 0; i < n; ++i) {
      int64_t c = cell_index(ps[i].x);
      cell_of[i] = c;
      if (c >= 0) cell_start[c + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) cell_start[c + 1] += cell_start[c];
    cell_items.assign(cell_start[nc], 0);
    std::vector<uint32_t> fill(cell_start.begin(), cell_start.end() - 1);
    for (size_t i = 0; i < n; ++i)
      if (cell_of[i] >= 0) cell_items[fill[cell_of[i]]++] = (uint32_t)i;
  }

  // src/grid.rs:48-87: visit candidate ids in the reference order.
  template <typename F>
  void for_candidates(const Particle<T>& p, F&& f) const {
    int32_t cc[3]; cell_coords(p.x, cc);
    for (int z = -1; z <= 1; ++z)
      for (int y = -1; y <= 1; ++y)
        for (int x = -1; x <= 1; ++x) {
          int32_t nc[3] = {cc[0] + x, cc[1] + y, cc[2] + z};  // i32 add (wraps in Rust release)
          for (int k = 0; k < 3; ++k) {
            if (!periodic[k]) continue;
            if (nc[k] < 0) nc[k] += gd[k];
            else if (nc[k] >= gd[k]) nc[k] -= gd[k];
          }
          if (nc[0] >= 0 && nc[0] < gd[0] && nc[1] >= 0 && nc[1] < gd[1] && nc[2] >= 0 && nc[2] < gd[2]) {
            size_t idx = (size_t)nc[0] + (size_t)nc[1] * gd[0] + (size_t)nc[2] * gd[0] * gd[1];
            for (uint32_t k = cell_start[idx]; k < cell_start[idx + 1]; ++k) f(cell_items[k]);
          }
        }
  }

  // Physical mode: every minimum-image pair within the cutoff, visited once.
  // Uses a private grid with cell >= largest cutoff; dims = floor(L/h) on
  // periodic axes (positions wrapped for binning), clamped on open axes.
  int pg[3];
  T ph[3];
  std::vector<uint32_t> pstart, pitems;
  std::vector<int32_t> pcell[3];
  void build_physical_grid(T maxcut) {
    size_t n = ps.size();
    V3<T> L = bmax - bmin;
    T Ls[3] = {L.x, L.y, L.z};
    for (int k = 0; k < 3; ++k) {
      T h = maxcut > T(0) ? maxcut : T(1);
      int64_t d = (int64_t)std::floor(Ls[k] / h);
      if (d < 1) d = 1;
      if (d > 4096) d = 4096;
      pg[k] = (int)d;
      ph[k] = Ls[k] / T(d);
      if (!periodic[k] && ph[k] < h) { ph[k] = h; }
    }
    T mins[3] = {bmin.x, bmin.y, bmin.z};
    for (int k = 0; k < 3; ++k) pcell[k].assign(n, 0);
    size_t nc = (size_t)pg[0] * pg[1] * pg[2];
    pstart.assign(nc + 1, 0);
    std::vector<uint32_t> lin(n);
    for (size_t i = 0; i < n; ++i) {
      T xs[3] = {ps[i].x.x, ps[i].x.y, ps[i].x.z};
      for (int k = 0; k < 3; ++k) {
        T q = xs[k];
        if (periodic[k]) { q = q - mins[k]; q = q - std::floor(q / Ls[k]) * Ls[k]; }
        else q = q - mins[k];
        int64_t c = (int64_t)std::floor(q / ph[k]);
        if (std::isnan(q)) c = 0;
        if (c < 0) c = 0;
        if (c >= pg[k]) c = pg[k] - 1;
        pcell[k][i] = (int32_t)c;
      }
      lin[i] = (uint32_t)(pcell[0][i] + (size_t)pcell[1][i] * pg[0] + (size_t)pcell[2][i] * pg[0] * pg[1]);
      pstart[lin[i] + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) pstart[c + 1] += pstart[c];
    pitems.assign(n, 0);
    std::vector<uint32_t> fill(pstart.begin(), pstart.end() - 1);
    for (size_t i = 0; i < n; ++i) pitems[fill[lin[i]]++] = (uint32_t)i;
  }
  template <typename F>
  void for_physical_candidates(size_t i, F&& f) const {
    int offs[3][3], no[3];
    for (int k = 0; k < 3; ++k) {
      int c = pcell[k][i];
      no[k] = 0;
      if (pg[k] >= 3) {
        for (int d = -1; d <= 1; ++d) {
          int q = c + d;
          if (periodic[k]) { if (q < 0) q += pg[k]; else if (q >= pg[k]) q -= pg[k]; }
          if (q < 0 || q >= pg[k]) continue;
          offs[k][no[k]++] = q;
        }
      } else {
        for (int q = 0; q < pg[k]; ++q) offs[k][no[k]++] = q;
      }
    }
    for (int a = 0; a < no[2]; ++a)
      for (int b = 0; b < no[1]; ++b)
        for (int c = 0; c < no[0]; ++c) {
          size_t idx = (size_t)offs[0][c] + (size_t)offs[1][b] * pg[0] + (size_t)offs[2][a] * pg[0] * pg[1];
          for (uint32_t k = pstart[idx]; k < pstart[idx + 1]; ++k) f(pitems[k]);
        }
  }

  void build_wall_cull(T rmax_) {
    const size_t nt = tris.size();
    cull_T = nt;
    cull_rmax = rmax_;
    const T grow = rmax_ * T(1.0001);
    std::vector<V3<T>> blo(nt), bhi(nt);
    V3<T> lo(T(1e30), T(1e30), T(1e30)), hi(T(-1e30), T(-1e30), T(-1e30));
    for (size_t t = 0; t < nt; ++t) {
      const Triangle<T>& tr = tris[t];
      V3<T> a(std::min(tr.v0.x, std::min(tr.v1.x, tr.v2.x)), std::min(tr.v0.y, std::min(tr.v1.y, tr.v2.y)),
              std::min(tr.v0.z, std::min(tr.v1.z, tr.v2.z)));
      V3<T> b(std::max(tr.v0.x, std::max(tr.v1.x, tr.v2.x)), std::max(tr.v0.y, std::max(tr.v1.y, tr.v2.y)),
              std::max(tr.v0.z, std::max(tr.v1.z, tr.v2.z)));
      blo[t] = V3<T>(a.x - grow, a.y - grow, a.z - grow);
      bhi[t] = V3<T>(b.x + grow, b.y + grow, b.z + grow);
      lo = V3<T>(std::min(lo.x, blo[t].x), std::min(lo.y, blo[t].y), std::min(lo.z, blo[t].z));
      hi = V3<T>(std::max(hi.x, bhi[t].x), std::max(hi.y, bhi[t].y), std::max(hi.z, bhi[t].z));
    }
    cull_lo = lo;
    T ext[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    T h = std::max(rmax_ * T(2), std::max(ext[0], std::max(ext[1], ext[2])) / T(512));
    if (!(h > T(0))) h = T(1);
    for (;;) {
      uint64_t tot = 1;
      for (int k = 0; k < 3; ++k) {
        cull_d[k] = std::max(1, (int)std::ceil(ext[k] / h) + 1);
        tot *= (uint64_t)cull_d[k];
      }
      if (tot <= ((uint64_t)1 << 23)) break;
      h = h * T(1.5);
    }
    cull_h = h;
    auto range = [&](T v, T o, int k) {
      int64_t c = (int64_t)std::floor((v - o) / h);
      return (int)std::max<int64_t>(0, std::min<int64_t>(c, cull_d[k] - 1));
    };
    const size_t nc = (size_t)cull_d[0] * cull_d[1] * cull_d[2];
    cull_start.assign(nc + 1, 0);
    auto each = [&](size_t t, auto&& f) {
      int a0 = range(blo[t].x, lo.x, 0), a1 = range(blo[t].y, lo.y, 1), a2 = range(blo[t].z, lo.z, 2);
      int b0 = range(bhi[t].x, lo.x, 0), b1 = range(bhi[t].y, lo.y, 1), b2 = range(bhi[t].z, lo.z, 2);
      for (int z = a2; z <= b2; ++z)
        for (int y = a1; y <= b1; ++y)
          for (int x = a0; x <= b0; ++x) f((size_t)x + (size_t)cull_d[0] * ((size_t)y + (size_t)cull_d[1] * z));
    };
    for (size_t t = 0; t < nt; ++t) each(t, [&](size_t c) { cull_start[c + 1]++; });
    for (size_t c = 0; c < nc; ++c) cull_start[c + 1] += cull_start[c];
    cull_items.assign(cull_start[nc], 0);
    std::vector<uint32_t> fill(cull_start.begin(), cull_start.end() - 1);
    for (size_t t = 0; t < nt; ++t) each(t, [&](size_t c) { cull_items[fill[c]++] = (uint32_t)t; });
  }
  // The culled triangle range of a centre: [s, e) into cull_items, empty
  // outside the grid (no grown box reaches there).
  void cull_range(V3<T> x, uint32_t& s, uint32_t& e) const {
    s = e = 0;
    T q[3] = {(x.x - cull_lo.x) / cull_h, (x.y - cull_lo.y) / cull_h, (x.z - cull_lo.z) / cull_h};
    int64_t c[3];
    for (int k = 0; k < 3; ++k) {
      if (!(q[k] >= T(0))) return;
      T f = std::floor(q[k]);
      if (f >= (T)cull_d[k]) return;
      c[k] = (int64_t)f;
    }
    const size_t idx = (size_t)c[0] + (size_t)cull_d[0] * ((size_t)c[1] + (size_t)cull_d[1] * c[2]);
    s = cull_start[idx];
    e = cull_start[idx + 1];
  }

  T max_cutoff() const {
    T rmax_ = 0;
    for (auto& p : ps) rmax_ = std::max(rmax_, p.r);
    T rs = rmax_ + rmax_;
    bool adh = (nmodel == N_JKR || nmodel == N_SJKR);
    return adh ? rs + rs * T(0.5) : rs;
  }

  Contact<T>& contact_entry(uint64_t key, std::unique_lock<std::mutex>& lk) {
    int s = (int)((key * 0x9E3779B97F4A7C15ull) >> 58) & (NSHARD - 1);
    lk = std::unique_lock<std::mutex>(cmut[s]);
    return cmap[s][key];
  }

  // One pair interaction seen from particle p (src/simulation.rs:327-461).
  // Returns false when outside the cutoff.
  inline bool pair_force(const Particle<T>& p, const Particle<T>& o, size_t i, size_t j, T es, T gs,
                         V3<T>& ftot, V3<T>& ttot, bool& excessive, Hist* hp, bool& in_contact, double& fs, double& ts) {
    V3<T> size = bmax - bmin;
    V3<T> d = p.x - o.x;
    if (periodic[0]) { if (d.x > size.x * T(0.5)) d.x = d.x - size.x; else if (d.x < -size.x * T(0.5)) d.x = d.x + size.x; }
    if (periodic[1]) { if (d.y > size.y * T(0.5)) d.y = d.y - size.y; else if (d.y < -size.y * T(0.5)) d.y = d.y + size.y; }
    if (periodic[2]) { if (d.z > size.z * T(0.5)) d.z = d.z - size.z; else if (d.z < -size.z * T(0.5)) d.z = d.z + size.z; }
    T d2 = d.length_squared();
    T rsum = p.r + o.r;
    T margin = (nmodel == N_JKR || nmodel == N_SJKR) ? rsum * T(0.5) : T(0);
    T cut = rsum + margin;
    in_contact = false;
    if (!(d2 < cut * cut)) return false;
    T dist = std::sqrt(d2);
    T overlap = rsum - dist;
    if (overlap > T(0.2) * std::min(p.r, o.r)) excessive = true;
    V3<T> n = dist > T(1e-6) ? d / dist : V3<T>(T(0), T(1), T(0));
    V3<T> ra = -n * p.r;
    V3<T> rb = n * o.r;
    V3<T> va = p.v + p.w.cross(ra);
    V3<T> vb = o.v + o.w.cross(rb);
    V3<T> rv = va - vb;
    T rs = effective_radius(p.r, o.r);
    T ms = effective_mass(p.m, o.m);
    tl_terms = 0.0;
    V3<T> fnv;
    switch (nmodel) {
      case N_HERTZ: fnv = hertzian(overlap, n, rv, es, rs, ms, pm.e); break;
      case N_LINEAR: { T kn = es * rs; T gn = T(0.5) * std::sqrt(ms * kn); fnv = linear_spring_dashpot(overlap, n, rv, kn, gn); } break;
      case N_HYSTERETIC: { T kn = es * rs; fnv = linear_spring_dashpot(overlap, n, V3<T>(), kn, T(0)); } break;
      case N_JKR: { T g = (pm.gamma + pm.gamma) * T(0.5); fnv = jkr(overlap, n, es, rs, g); } break;
      default: { T g = (pm.gamma + pm.gamma) * T(0.5); fnv = sjkr(overlap, n, rv, es, rs, g); } break;
    }
    T fn = fnv.length();
    V3<T> ft;
    if (tmodel == T_COULOMB) {
      ft = coulomb(fn, rv, n, pm.mu);
      if (mode == MODE_PARITY && keep_contact_map) {
        uint64_t key = i < j ? (i << 32 | j) : (j << 32 | i);
        std::unique_lock<std::mutex> lk;
        contact_entry(key, lk).age += 1;
      }
    } else if (mode == MODE_PARITY) {
      uint64_t key = i < j ? (i << 32 | j) : (j << 32 | i);
      std::unique_lock<std::mutex> lk;
      Contact<T>& c = contact_entry(key, lk);
      c.age += 1;
      if (tmodel == T_MINDLIN) {
        T kt = T(8) * gs * std::sqrt(rs * overlap);
        ft = linear_spring_coulomb(fn, rv, n, c.xi, kt, pm.mu, dt);
      } else {
        T kt = gs * rs;
        ft = linear_spring_coulomb(fn, rv, n, c.xi, kt, pm.mu, dt);
      }
    } else {
      // physical mode: directed history hp (already looked up), reset out of contact
      if (overlap > T(0)) {
        T kt = tmodel == T_MINDLIN ? T(8) * gs * std::sqrt(rs * overlap) : gs * rs;
        V3<T> xi = hp->xi;
        xi = xi - xi.dot(n) * n;  // keep the spring in the current tangent plane
        ft = linear_spring_coulomb(fn, rv, n, xi, kt, pm.mu, dt);
        hp->xi = xi;
        in_contact = true;
      }
    }
    V3<T> fc = fnv + ft;
    ftot += fc;
    V3<T> tc = ra.cross(fc);
    ttot += tc;
    fs += tl_terms;
    ts += (double)p.r * tl_terms;  // |r_a| x the force scale: the rounding scale of r_a x f
    return true;
  }

  void step() {
    const size_t n0 = ps.size();
    bool par = n0 >= 256;  // thread fork/join costs more than it saves on tiny systems
    // 0. boundaries (src/simulation.rs:176-219)
    V3<T> size = bmax - bmin;
    if (periodic[0] || periodic[1] || periodic[2]) {
#pragma omp parallel for schedule(static) if (par)
      for (long i = 0; i < (long)n0; ++i) {
        Particle<T>& p = ps[i];
        if (periodic[0]) { if (p.x.x < bmin.x) p.x.x = p.x.x + size.x; else if (p.x.x >= bmax.x) p.x.x = p.x.x - size.x; }
        if (periodic[1]) { if (p.x.y < bmin.y) p.x.y = p.x.y + size.y; else if (p.x.y >= bmax.y) p.x.y = p.x.y - size.y; }
        if (periodic[2]) { if (p.x.z < bmin.z) p.x.z = p.x.z + size.z; else if (p.x.z >= bmax.z) p.x.z = p.x.z - size.z; }
      }
    }
    {
      size_t w = 0;
      for (size_t i = 0; i < n0; ++i) {
        const Particle<T>& p = ps[i];
        bool keep = (periodic[0] || (p.x.x >= bmin.x - T(1) && p.x.x <= bmax.x + T(1))) &&
                    (periodic[1] || (p.x.y >= bmin.y - T(1))) &&
                    (periodic[2] || (p.x.z >= bmin.z - T(1) && p.x.z <= bmax.z + T(1)));
        if (keep) {
          if (w != i) { ps[w] = ps[i]; hist[w] = std::move(hist[i]); }
          ++w;
        }
      }
      ps.resize(w);
      hist.resize(w);
    }
    const size_t n = ps.size();
    // 1. first half update (src/simulation.rs:232-263)
#pragma omp parallel for schedule(static) if (par)
    for (long i = 0; i < (long)n; ++i) {
      Particle<T>& p = ps[i];
      if (p.fixed) continue;
      V3<T> dv = (T(0.5) * p.a) * dt;
      V3<T> yv = dv - p.vres;
      V3<T> tv = p.v + yv;
      p.vres = (tv - p.v) - yv;
      p.v = tv;
      V3<T> dx = p.v * dt;
      V3<T> yx = dx - p.xres;
      V3<T> tx = p.x + yx;
      p.xres = (tx - p.x) - yx;
      p.x = tx;
      T inertia = T(0.4) * p.m * p.r * p.r;
      V3<T> aa = p.tau / inertia;
      V3<T> dw = (T(0.5) * aa) * dt;
      V3<T> yw = dw - p.wres;
      V3<T> tw = p.w + yw;
      p.wres = (tw - p.w) - yw;
      p.w = tw;
    }
    // 2. force reset (src/simulation.rs:265-271)
#pragma omp parallel for schedule(static) if (par)
    for (long i = 0; i < (long)n; ++i) { ps[i].a = gravity; ps[i].tau = V3<T>(); }
    // broad phase
    if (mode == MODE_PARITY) { if (grid_dims() != 0) { fprintf(stderr, "oracle: grid too large\n"); return; } build_grid(); }
    else build_physical_grid(max_cutoff());
    if (wall_cull && !tris.empty()) {
      T rm = T(0);
      for (const Particle<T>& p : ps) rm = std::max(rm, p.r);
      if (cull_T != tris.size() || rm > cull_rmax) build_wall_cull(rm);
    }
    // 3. per-particle force gather (src/simulation.rs:317-526)
    T es = effective_youngs(pm.E, pm.nu, pm.E, pm.nu);
    T gs = mode == MODE_PARITY ? T(0) : physical_shear(pm.E, pm.nu, pm.E, pm.nu);
    T ew = effective_youngs(pm.E, pm.nu, wm.E, wm.nu);
    lastF.assign(n, V3<T>());
    lastT.assign(n, V3<T>());
    lastFS.assign(n, 0.0);
    lastTS.assign(n, 0.0);
    pair_i.clear(); pair_j.clear();
    int excessive_any = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : excessive_any) if (par)
    for (long il = 0; il < (long)n; ++il) {
      size_t i = (size_t)il;
      const Particle<T>& p = ps[i];
      V3<T> ftot, ttot;
      double fs = 0.0, ts = 0.0;
      bool excessive = false;
      std::vector<Hist> nh;
      std::vector<uint64_t> li, lj;
      if (mode == MODE_PARITY) {
        for_candidates(p, [&](uint32_t j) {
          if (j == i) return;
          bool ic;
          if (pair_force(p, ps[j], i, j, es, gs, ftot, ttot, excessive, nullptr, ic, fs, ts) && record_pairs) {
            li.push_back(i); lj.push_back(j);
          }
        });
      } else {
        const std::vector<Hist>& old = hist[i];
        for_physical_candidates(i, [&](uint32_t j) {
          if (j == i) return;
          Hist h{ps[j].tag, V3<T>()};
          auto it = std::lower_bound(old.begin(), old.end(), h.tag, [](const Hist& a, uint64_t t) { return a.tag < t; });
          if (it != old.end() && it->tag == h.tag) h.xi = it->xi;
          bool ic;
          if (pair_force(p, ps[j], i, j, es, gs, ftot, ttot, excessive, &h, ic, fs, ts)) {
            if (record_pairs) { li.push_back(i); lj.push_back(j); }
            if (ic) nh.push_back(h);
          }
        });
      }
      // particle-mesh (src/simulation.rs:464-523)
      uint32_t ts0 = 0, ts1 = (uint32_t)tris.size();
      if (wall_cull && !tris.empty()) cull_range(p.x, ts0, ts1);
      for (uint32_t tt = ts0; tt < ts1; ++tt) {
        const Triangle<T>& tr = tris[wall_cull ? cull_items[tt] : tt];
        T pen; V3<T> nrm, cp;
        if (!intersect_sphere(tr, p.x, p.r, pen, nrm, &cp)) continue;
        if (pen > T(0.2) * p.r) excessive = true;
        V3<T> ra = -nrm * p.r;
        V3<T> va = p.v + p.w.cross(ra);
        V3<T> rv = va;
        if (tr.motion >= 0) {  // extension: the wall surface moves with V + W x (cp - C)
          const WallMotion& M = motions[tr.motion];
          const V3<T> arm = cp - V3<T>((T)M.c[0], (T)M.c[1], (T)M.c[2]);
          const V3<T> vw = V3<T>((T)M.v[0], (T)M.v[1], (T)M.v[2]) + V3<T>((T)M.w[0], (T)M.w[1], (T)M.w[2]).cross(arm);
          rv = rv - vw;
        }
        T rs = p.r, ms = p.m;
        tl_terms = 0.0;
        V3<T> fnv;
        switch (nmodel) {
          case N_HERTZ: fnv = hertzian(pen, nrm, rv, ew, rs, ms, pm.e); break;
          case N_LINEAR: { T kn = ew * rs; T gn = T(0.5) * std::sqrt(ms * kn); fnv = linear_spring_dashpot(pen, nrm, rv, kn, gn); } break;
          case N_HYSTERETIC: { T kn = ew * rs; fnv = linear_spring_dashpot(pen, nrm, rv, kn, T(0)); } break;
          case N_JKR: { T g = (pm.gamma + wm.gamma) * T(0.5); fnv = jkr(pen, nrm, ew, rs, g); } break;
          default: { T g = (pm.gamma + wm.gamma) * T(0.5); fnv = sjkr(pen, nrm, rv, ew, rs, g); } break;
        }
        T fn = fnv.length();
        V3<T> ft = coulomb(fn, rv, nrm, pm.mu);
        V3<T> fc = fnv + ft;
        ftot += fc;
        V3<T> tc = ra.cross(fc);
        ttot += tc;
        fs += tl_terms;
        ts += (double)p.r * tl_terms;
      }
      lastF[i] = ftot;
      lastT[i] = ttot;
      lastFS[i] = fs;
      lastTS[i] = ts;
      if (excessive) excessive_any = 1;
      if (mode == MODE_PHYSICAL) {
        std::sort(nh.begin(), nh.end(), [](const Hist& a, const Hist& b) { return a.tag < b.tag; });
        hist[i].swap(nh);  // only thread i writes hist[i]; readers use ps[j].tag, not hist[j]
      }
      if (record_pairs && !li.empty()) {
        std::lock_guard<std::mutex> g(pair_mut);
        pair_i.insert(pair_i.end(), li.begin(), li.end());
        pair_j.insert(pair_j.end(), lj.begin(), lj.end());
      }
    }
    if (excessive_any) {
      ++overlap_warnings;
      if (warn_stderr) fprintf(stderr, "Warning: Excessive particle overlap detected (>20%% of radius). Simulation may be unstable.\n");
    }
    // apply (src/simulation.rs:532-536)
#pragma omp parallel for schedule(static) if (par)
    for (long i = 0; i < (long)n; ++i) {
      Particle<T>& p = ps[i];
      p.a += lastF[i] / p.m;
      p.tau += lastT[i];
    }
    // 4. second half update (src/simulation.rs:541-561)
#pragma omp parallel for schedule(static) if (par)
    for (long i = 0; i < (long)n; ++i) {
      Particle<T>& p = ps[i];
      if (p.fixed) continue;
      V3<T> dv = (T(0.5) * p.a) * dt;
      V3<T> yv = dv - p.vres;
      V3<T> tv = p.v + yv;
      p.vres = (tv - p.v) - yv;
      p.v = tv;
      T inertia = T(0.4) * p.m * p.r * p.r;
      V3<T> aa = p.tau / inertia;
      V3<T> dw = (T(0.5) * aa) * dt;
      V3<T> yw = dw - p.wres;
      V3<T> tw = p.w + yw;
      p.wres = (tw - p.w) - yw;
      p.w = tw;
    }
    ++steps_done;
  }
};

struct Handle {
  int prec;  // 32 or 64
  Base* sim;
};

}  // namespace orc

using namespace orc;

template <typename F>
static auto dispatch(Handle* h, F&& f) {
  if (h->prec == 32) return f(static_cast<Sim<float>*>(h->sim));
  return f(static_cast<Sim<double>*>(h->sim));
}

extern "C" {

// Oracle C ABI (test and baseline use only).
void* orc_create(int prec, double dt, const double* mn, const double* mx) {
  Handle* h = new Handle;
  h->prec = prec == 32 ? 32 : 64;
  if (h->prec == 32)
    h->sim = new Sim<float>((float)dt, V3<float>((float)mn[0], (float)mn[1], (float)mn[2]),
                            V3<float>((float)mx[0], (float)mx[1], (float)mx[2]));
  else
    h->sim = new Sim<double>(dt, V3<double>(mn[0], mn[1], mn[2]), V3<double>(mx[0], mx[1], mx[2]));
  return h;
}
void orc_destroy(void* hv) {
  Handle* h = (Handle*)hv;
  if (!h) return;
  delete h->sim;
  delete h;
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}
int orc_get_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_add_particle(void* hv, double x, double y, double z, double r, double m, int fixed) {
  dispatch((Handle*)hv, [&](auto* s) {
    using T = decltype(s->dt);
    s->add_particle(V3<T>((T)x, (T)y, (T)z), (T)r, (T)m, fixed != 0);
    return 0;
  });
}
// Bulk form of orc_add_particle: xyz 3n doubles, r and m n doubles, fixed n bytes (may be null).
void orc_add_particles(void* hv, long n, const double* xyz, const double* r, const double* m, const unsigned char* fixed) {
  dispatch((Handle*)hv, [&](auto* s) {
    using T = decltype(s->dt);
    s->ps.reserve(s->ps.size() + (size_t)n);
    for (long i = 0; i < n; ++i)
      s->add_particle(V3<T>((T)xyz[3 * i], (T)xyz[3 * i + 1], (T)xyz[3 * i + 2]), (T)r[i], (T)m[i],
                      fixed ? fixed[i] != 0 : false);
    return 0;
  });
}
// Benchmark-side variant: cull the wall loop by a triangle grid (same contacts,
// same order as the every-triangle loop; off by default).
void orc_set_wall_cull(void* hv, int on) {
  dispatch((Handle*)hv, [&](auto* s) { s->wall_cull = on != 0; s->cull_T = 0; return 0; });
}
// v: 9 doubles per triangle (v0,v1,v2), nrm: 3 doubles per triangle
void orc_add_triangles(void* hv, const double* v, const double* nrm, long nt) {
  dispatch((Handle*)hv, [&](auto* s) {
    using T = decltype(s->dt);
    for (long k = 0; k < nt; ++k) {
      Triangle<T> t;
      const double* q = v + 9 * k;
      t.v0 = V3<T>((T)q[0], (T)q[1], (T)q[2]);
      t.v1 = V3<T>((T)q[3], (T)q[4], (T)q[5]);
      t.v2 = V3<T>((T)q[6], (T)q[7], (T)q[8]);
      t.n = V3<T>((T)nrm[3 * k], (T)nrm[3 * k + 1], (T)nrm[3 * k + 2]);
      s->tris.push_back(t);
    }
    return 0;
  });
}
// Extension: triangles whose surface moves with V + W x (p - C).
void orc_add_triangles_moving(void* hv, const double* v, const double* nrm, long nt, const double* c9) {
  dispatch((Handle*)hv, [&](auto* s) {
    using T = decltype(s->dt);
    WallMotion m;
    for (int k = 0; k < 3; ++k) {
      m.c[k] = c9[k];
      m.w[k] = c9[3 + k];
      m.v[k] = c9[6 + k];
    }
    s->motions.push_back(m);
    const int id = (int)s->motions.size() - 1;
    for (long k = 0; k < nt; ++k) {
      Triangle<T> t;
      const double* q = v + 9 * k;
      t.v0 = V3<T>((T)q[0], (T)q[1], (T)q[2]);
      t.v1 = V3<T>((T)q[3], (T)q[4], (T)q[5]);
      t.v2 = V3<T>((T)q[6], (T)q[7], (T)q[8]);
      t.n = V3<T>((T)nrm[3 * k], (T)nrm[3 * k + 1], (T)nrm[3 * k + 2]);
      t.motion = id;
      s->tris.push_back(t);
    }
    return 0;
  });
}
void orc_set_material(void* hv, int wall, double E, double nu, double rho, double mu, double e, double gamma) {
  dispatch((Handle*)hv, [&](auto* s) {
    using T = decltype(s->dt);
    Material<T> m{(T)E, (T)nu, (T)rho, (T)mu, (T)e, (T)gamma};
    if (wall) s->wm = m; else s->pm = m;
    return 0;
  });
}
void orc_set_models(void* hv, int normal, int tangential) {
  dispatch((Handle*)hv, [&](auto* s) { s->nmodel = normal; s->tmodel = tangential; return 0; });
}
void orc_set_periodic(void* hv, int x, int y, int z) {
  dispatch((Handle*)hv, [&](auto* s) { s->periodic[0] = x; s->periodic[1] = y; s->periodic[2] = z; return 0; });
}
void orc_set_mode(void* hv, int mode) { dispatch((Handle*)hv, [&](auto* s) { s->mode = mode; return 0; }); }
void orc_set_cell_size(void* hv, double h) {
  dispatch((Handle*)hv, [&](auto* s) { using T = decltype(s->dt); s->cell = (T)h; return 0; });
}
void orc_set_gravity(void* hv, double gx, double gy, double gz) {
  dispatch((Handle*)hv, [&](auto* s) { using T = decltype(s->dt); s->gravity = V3<T>((T)gx, (T)gy, (T)gz); return 0; });
}
void orc_set_options(void* hv, int record_pairs, int keep_contact_map, int warn_stderr) {
  dispatch((Handle*)hv, [&](auto* s) {
    s->record_pairs = record_pairs != 0;
    s->keep_contact_map = keep_contact_map != 0;
    s->warn_stderr = warn_stderr;
    return 0;
  });
}
void orc_step(void* hv, long nsteps) {
  dispatch((Handle*)hv, [&](auto* s) { for (long k = 0; k < nsteps; ++k) s->step(); return 0; });
}
long orc_count(void* hv) { return dispatch((Handle*)hv, [&](auto* s) { return (long)s->ps.size(); }); }
long orc_overlap_warnings(void* hv) { return dispatch((Handle*)hv, [&](auto* s) { return (long)s->overlap_warnings; }); }
long orc_contact_map_size(void* hv) {
  return dispatch((Handle*)hv, [&](auto* s) {
    long k = 0;
    for (int q = 0; q < s->NSHARD; ++q) k += (long)s->cmap[q].size();
    return k;
  });
}

// State transfer. Any pointer may be null. Vectors are 3 doubles per particle.
// which: 0 x, 1 v, 2 a, 3 w, 4 tau, 5 xres, 6 vres, 7 wres
void orc_get_vec(void* hv, int which, double* out) {
  dispatch((Handle*)hv, [&](auto* s) {
    for (size_t i = 0; i < s->ps.size(); ++i) {
      auto& p = s->ps[i];
      auto v = which == 0 ? p.x : which == 1 ? p.v : which == 2 ? p.a : which == 3 ? p.w : which == 4 ? p.tau
             : which == 5 ? p.xres : which == 6 ? p.vres : p.wres;
      out[3 * i] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z;
    }
    return 0;
  });
}
void orc_set_vec(void* hv, int which, const double* in) {
  dispatch((Handle*)hv, [&](auto* s) {
    using T = decltype(s->dt);
    for (size_t i = 0; i < s->ps.size(); ++i) {
      auto& p = s->ps[i];
      V3<T> v((T)in[3 * i], (T)in[3 * i + 1], (T)in[3 * i + 2]);
      switch (which) {
        case 0: p.x = v; break; case 1: p.v = v; break; case 2: p.a = v; break; case 3: p.w = v; break;
        case 4: p.tau = v; break; case 5: p.xres = v; break; case 6: p.vres = v; break; default: p.wres = v; break;
      }
    }
    return 0;
  });
}
// scalars: 0 radius, 1 mass, 2 fixed, 3 tag
void orc_get_scalar(void* hv, int which, double* out) {
  dispatch((Handle*)hv, [&](auto* s) {
    for (size_t i = 0; i < s->ps.size(); ++i) {
      auto& p = s->ps[i];
      out[i] = which == 0 ? (double)p.r : which == 1 ? (double)p.m : which == 2 ? (double)p.fixed : (double)p.tag;
    }
    return 0;
  });
}
// Per-particle (f_total, torque_total) of the last step, before division by mass.
void orc_last_forces(void* hv, double* F, double* Tq) {
  dispatch((Handle*)hv, [&](auto* s) {
    for (size_t i = 0; i < s->lastF.size(); ++i) {
      F[3 * i] = s->lastF[i].x; F[3 * i + 1] = s->lastF[i].y; F[3 * i + 2] = s->lastF[i].z;
      Tq[3 * i] = s->lastT[i].x; Tq[3 * i + 1] = s->lastT[i].y; Tq[3 * i + 2] = s->lastT[i].z;
    }
    return 0;
  });
}
// Per-particle force scale of the last step: the sum over contacts of the
// magnitudes of each law's additive terms (and r times it for torques).
void orc_last_force_scale(void* hv, double* FS, double* TS) {
  dispatch((Handle*)hv, [&](auto* s) {
    for (size_t i = 0; i < s->lastFS.size(); ++i) { FS[i] = s->lastFS[i]; TS[i] = s->lastTS[i]; }
    return 0;
  });
}
// Reference-grid state of the last step: dims, per-particle cell (-1 when not
// inserted) and the flattened cell contents (the stable cell order).
void orc_grid_dims(void* hv, int* d) { dispatch((Handle*)hv, [&](auto* s) { d[0] = s->gd[0]; d[1] = s->gd[1]; d[2] = s->gd[2]; return 0; }); }
long orc_grid_items(void* hv, long* cell_of, long* order) {
  return dispatch((Handle*)hv, [&](auto* s) {
    for (size_t i = 0; i < s->cell_of.size(); ++i) cell_of[i] = (long)s->cell_of[i];
    for (size_t k = 0; k < s->cell_items.size(); ++k) order[k] = (long)s->cell_items[k];
    return (long)s->cell_items.size();
  });
}
// Compute the reference grid for the current positions without stepping.
int orc_grid_now(void* hv) {
  return dispatch((Handle*)hv, [&](auto* s) { if (s->grid_dims() != 0) return -1; s->build_grid(); return 0; });
}
long orc_pair_count(void* hv) { return dispatch((Handle*)hv, [&](auto* s) { return (long)s->pair_i.size(); }); }
void orc_pairs(void* hv, long* pi, long* pj) {
  dispatch((Handle*)hv, [&](auto* s) {
    for (size_t k = 0; k < s->pair_i.size(); ++k) { pi[k] = (long)s->pair_i[k]; pj[k] = (long)s->pair_j[k]; }
    return 0;
  });
}
// Single-triangle query, for the mesh known-answer test (src/mesh.rs:146-172).
int orc_triangle_query(int prec, const double* v9, const double* n3, const double* c, double r, double* pen, double* nrm) {
  if (prec == 32) {
    Triangle<float> t{V3<float>(v9[0], v9[1], v9[2]), V3<float>(v9[3], v9[4], v9[5]), V3<float>(v9[6], v9[7], v9[8]),
                      V3<float>(n3[0], n3[1], n3[2])};
    float p; V3<float> n;
    bool hit = intersect_sphere(t, V3<float>(c[0], c[1], c[2]), (float)r, p, n);
    if (hit) { *pen = p; nrm[0] = n.x; nrm[1] = n.y; nrm[2] = n.z; }
    return hit;
  }
  Triangle<double> t{V3<double>(v9[0], v9[1], v9[2]), V3<double>(v9[3], v9[4], v9[5]), V3<double>(v9[6], v9[7], v9[8]),
                     V3<double>(n3[0], n3[1], n3[2])};
  double p; V3<double> n;
  bool hit = intersect_sphere(t, V3<double>(c[0], c[1], c[2]), r, p, n);
  if (hit) { *pen = p; nrm[0] = n.x; nrm[1] = n.y; nrm[2] = n.z; }
  return hit;
}
// Scalar force-law probes (prec 64), for unit tests of the laws.
double orc_jkr_force(double overlap, double es, double rs, double gamma) {
  return jkr<double>(overlap, V3<double>(1, 0, 0), es, rs, gamma).x;
}
// The contact radius the reference's Newton loop ends on, and its loop count.
double orc_jkr_radius(double overlap, double es, double rs, double gamma, int* iters) {
  return jkr_radius<double>(overlap, es, rs, gamma, iters);
}
}
