// Device-side data layout and parameters of the DEM step.
//
// Particles live in HBM as structure-of-arrays in "slots": after each
// neighbour-list rebuild the slots are re-ordered by fine cell, so particles
// that interact sit close together in memory. Every per-slot array exists in
// two banks; a rebuild gathers bank b into bank 1-b and flips `Ctrl::bank`,
// so no kernel ever reads a slot another thread is writing.
//
// Each 32-byte record packs what one gather needs (x,y,z,radius), (v,mass),
// (omega, reference-grid cell code): a neighbour costs three aligned 32-byte
// sectors.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rp {

struct alignas(32) D4 {
  double x, y, z, w;
};

// PF_WALLFAR (set at each list rebuild, with wall_far_ok): no triangle within
// reach of the slot until the next rebuild, so the filter skips its walls
enum : uint32_t { PF_FIXED = 1u, PF_DEAD = 2u, PF_WALLFAR = 4u };

enum : unsigned { ST_OVERLAP = 1u, ST_NAN = 2u, ST_NLIST_GROW = 4u, ST_WALL_GROW = 8u };

// Device control block: written by kernels, read by the host after a chunk.
struct Ctrl {
  int bank;                       // bank holding the current state
  int rebuild;                    // rebuild requested for the current step
  int halt;                       // HALT_* bits: a buffer outgrew its capacity; later kernels of the chunk no-op
  int overlap_flag;               // overlap > 20 % seen in the current step
  unsigned int status;            // sticky ST_* bits
  unsigned int max_count;         // longest neighbour list seen by the last build
  unsigned long long removed;     // slots marked dead since the last compaction
  unsigned long long steps_done;  // completed steps
  unsigned long long rebuilds;    // completed list rebuilds
  unsigned long long overlap_steps;
  int pending;                    // the last completed step still owes its second half kick
  unsigned int wall_need;         // wall candidates a halted filter wanted room for
  unsigned long long target;      // device step loop: run while steps_done < target
  unsigned long long iters;       // device step loop iterations (bounded by target + 4)
  // learned JKR tallies (pair evaluations): network/certified-solver results
  // accepted, certified zeros, reference-Newton fallbacks, network rows, FP32
  // Newton steps, closed-form walks
  unsigned long long jkr_count[6];
};

struct Material {
  double E, nu, rho, mu, e, gamma;
};

// Constants of the pair and wall laws for one group of particles. A group is
// an independent bed: its particles interact only with each other and with
// the triangles of the group (or of GROUP_ALL), under the group's particle
// material. Group 0 is the simulation's particle material; a simulation with
// one group is exactly the reference's single-material simulation.
struct Law {
  double es_pp, es_pw, gs_pp;  // effective Young's moduli (pair, wall) and shear modulus (pair)
  double gamma_pp, gamma_pw;   // combined surface energies
  double beta_abs;             // |ln e / sqrt(ln^2 e + pi^2)| of the particle restitution (host libm)
  double mu;                   // particle friction, used for pairs and walls (src/simulation.rs:489)
  double jkr_C;                // 8 pi gamma / E* of pairs, as src/physics.rs:165 forms it
  float jkr_Cf, pad_;
};
constexpr uint32_t GROUP_ALL = 0xFFFFFFFFu;
// Ctrl::halt bits: a neighbour list outgrew its capacity (list rebuild), the
// wall candidates outgrew their arena (contact filter)
constexpr int HALT_LISTS = 1;
constexpr int HALT_WALLS = 2;

// A rigid surface velocity V + W x (p - C) of a set of triangles whose geometry
// stays put (a surface of revolution turning about its own axis, a belt). The
// reference's walls are static; a wall with a motion enters the contact's
// relative velocity at the contact point.
struct WallMotion {
  double c[3], w[3], v[3];
};
constexpr uint32_t NO_MOTION = 0xFFFFFFFFu;

struct Bank {
  D4* xr;    // position, radius
  D4* vm;    // velocity, mass
  D4* wc;    // angular velocity, reference-grid cell code (bit pattern in .w)
  D4* acc;   // acceleration
  D4* tq;    // torque
  D4* xres;  // Kahan residuals (src/particle.rs:12-18)
  D4* vres;
  D4* wres;
  uint32_t* flags;  // PF_*
  uint32_t* tag;    // insertion number (stable identity)
  float4* xref;     // position at the last list build (.w unused)
  float4* xf;       // FP32 mirror of (position, radius) for the pair pretest
  uint32_t* nbr;    // neighbour rows, cap entries per slot
  uint32_t* ncnt;   // row lengths
  double* hist;     // physical-mode tangential spring per row entry: 3 planes of N*cap
  // physical mode: bit m set when the spring of row entry m (< 64) may hold a
  // value other than +0 (entries past 64 are always treated as live)
  unsigned long long* hmask;
  uint32_t* grp;    // group (independent bed) of the slot
};

// Triangle record with the per-triangle constants of src/mesh.rs:45-62
// precomputed (same operations, so the values are bit-identical).
struct TriRec {
  double v0[3], e0[3], e1[3], n[3];
  double a, b, c, det, denom;
  uint32_t group;   // the group whose particles touch it (GROUP_ALL: every particle)
  uint32_t motion;  // index into StepParams::motions, NO_MOTION for a static wall
  float4 plane;  // unit normal from the vertices and n.v0, FP32 (zero for a degenerate triangle)
  float4 bound;  // .x = largest |vertex coordinate| (scales the FP32 plane-test error)
  float4 edge[3];  // per edge: in-plane outward unit normal m and m.(edge start); (0,0,0,1e30) if degenerate
};

// A contact candidate kept by the filter: neighbour slot, row position and
// the reference's visit counts from both ends (m | vis_ij << 16 | vis_ji << 24,
// visit counts <= 27), bit 31 set when the pair is queued for the JKR network.
constexpr uint32_t CREC_NET = 0x80000000u;
__host__ __device__ __forceinline__ int crec_vji(uint32_t mv) { return (int)((mv >> 24) & 0x7Fu); }
struct CRec {
  uint32_t j;
  uint32_t mv;
};

struct MlpInfer;

struct StepParams {
  int n;  // slots
  int cap;
  int force_path;  // 0: contact-parallel (default), 1: one thread per particle
  // launch shapes of the force pass (chosen by the autotuner): threads per
  // block of the filter, pair and accumulate kernels (<= 256), and the
  // largest grid of their grid-stride loops
  int bs_filter, bs_force, bs_accum, grid_cap;
  int nsm;  // multiprocessors of the device (sizes the default grids)
  // contact-parallel buffers (recomputed every step)
  CRec* crec;       // n*cap records, row k at k*cap
  uint32_t* ccnt;   // records per particle
  uint32_t* aorder; // slots in the order k_accumulate visits them (a permutation within tiles of 256)
  uint2* warena;    // wall candidates (slot, triangle); a particle's at woff, in mesh order; min(ctot[4], wcap)
  double* wres;     // per wall candidate: force (3) and torque (3) on the particle
  uint8_t* wok;     // per wall candidate: 1 when the sphere touches the triangle
  uint32_t* woff;   // first wall candidate of slot k
  uint32_t* wcnt;   // wall candidates of slot k
  uint32_t wcap;    // wall candidate capacity
  uint32_t* coff;   // first result slot of particle k (its ccnt results are contiguous)
  uint32_t* clist;  // compact list of evaluating record slots
  uint32_t* ctot;   // [0] records, [1] evaluating records, [2] network queue, [3] deferred pairs, [4] wall candidates
  uint32_t* jfb;    // evaluating indices deferred to the reference-Newton pass (null: no deferral)
  double* cres;     // per record: force (3) and torque (3) on the row's particle
  float* cresf;     // the same buffer as FP32 records (the mixed form: its pair forces are FP32 values)
  int nmodel, tmodel, mode, prec;
  int periodic[3];
  int debug;
  double dt;
  double bmin[3], bmax[3], bsize[3];
  float bsizef[3];  // (float)bsize: FP32 kernels take no double-to-float conversion per use
  // per axis, an FP32 interval whose interior (on the FP32 mirror) proves the
  // FP64 position needs no periodic wrap (periodic axes) or is kept (open axes)
  float inner_lo[3], inner_hi[3];
  uint32_t bq_hi[3]; // high word of the bits of bsize/4: |d| has a smaller high word => |d| < bsize/4
  double gravity[3];
  Material pm, wm;
  Law law;             // group 0 (the host's copy; kernels read glaw)
  int ngroups;         // 1: no group array is read
  const Law* glaw;     // per group, device array of ngroups entries
  // reference grid (parity-mode visit rule)
  double href, inv_href;
  int rdims[3];
  int same_cell_visits;  // ref_visits(c, c) for a cell c inside the grid (3 per periodic axis of one cell, else 1)
  // fine grid (neighbour search)
  double fmin[3], fcell[3];
  double finv[3], binv[3];  // 1 / fcell, 1 / bsize
  float fcellf[3], binvf[3];
  float rmaxf;              // largest radius (culls the cells of the list search)
  float xbound;             // largest |box bound| + 1 (rounding margins of periodic images)
  int fdims[3];
  uint32_t fncells;
  double skin;
  float list_scale;  // 1 + relative margin of the FP32 list test
  int pretest;       // FP32 pair pretest enabled (off when a periodic length < 4 cutoffs)
  float lmax;        // largest periodic length (enters the pretest rounding bound)
  // triangles
  int ntri;
  const TriRec* tri;
  double tmin[3], tcell;
  float tminf[3], tinvf;  // FP32 lookup: cell = floor((x - tmin) * (1/tcell))
  int tdims[3];
  const uint32_t* tstart;
  const uint32_t* titems;
  const WallMotion* motions;
  int wall_far_ok;       // the triangle-grid cell exceeds half the skin: PF_WALLFAR is set and read
  float wall_far_gap;    // half the skin with margin: the distance a slot keeps from a periodic face
  // JKR solver for particle pairs: 0 the reference's Newton, 1 certificates +
  // network + polish, 2 certificates + FP32 Newton from the reference's start
  int jkr_solver;
  float jdom_lo[4], jdom_hi[4];  // raw-feature range of the training set
  const MlpInfer* mlp;
  uint2* jq;        // network queue: (evaluating index, record slot); length ctot[2]
  float* jguess;    // per evaluating index: predicted a/R* (NaN = outside the training range)
  // diagnostics
  double* dbgF;
  double* dbgT;
  uint8_t* dbgMult;
  Ctrl* ctrl;
  Bank bank[2];
};

// The law constants of slot k's group (a value copy: kernel parameters are
// never addressed).
__device__ __forceinline__ Law law_of(const StepParams& P, const Bank& B, int k) {
  return P.glaw[P.ngroups > 1 ? B.grp[k] : 0u];
}

// ---- non-contracted double arithmetic (matches the oracle's rounding) ----
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Rust `as i32` from a float: saturating, NaN -> 0.
__device__ __forceinline__ int32_t sat_i32(double f) {
  if (f != f) return 0;
  if (f <= -2147483648.0) return INT32_MIN;
  if (f >= 2147483647.0) return INT32_MAX;
  return (int32_t)f;
}

// Reference-grid coordinates packed into 63 bits (21 bits per axis, signed,
// saturated at +-(2^20-1); dims are capped below that on the host so the
// saturation never changes a visit decision).
__device__ __forceinline__ unsigned long long pack_code(int32_t cx, int32_t cy, int32_t cz) {
  const int32_t L = (1 << 20) - 1;
  cx = cx < -L ? -L : (cx > L ? L : cx);
  cy = cy < -L ? -L : (cy > L ? L : cy);
  cz = cz < -L ? -L : (cz > L ? L : cz);
  return ((unsigned long long)(uint32_t)(cx & 0x1FFFFF)) | ((unsigned long long)(uint32_t)(cy & 0x1FFFFF) << 21) |
         ((unsigned long long)(uint32_t)(cz & 0x1FFFFF) << 42);
}
__device__ __forceinline__ int32_t code_axis(unsigned long long c, int k) {
  int32_t v = (int32_t)((c >> (21 * k)) & 0x1FFFFF);
  return (v << 11) >> 11;  // sign-extend 21 bits
}

// floor(d / h) with the correctly rounded quotient, from the product with the
// rounded reciprocal: d * rd(1/h) lies within 3 u |d/h| (u = 2^-53) of rd(d/h),
// so the two floors agree unless the product is within 8 u |q| of an integer;
// only then is the division itself evaluated.
__device__ __forceinline__ double floor_div_exact(double d, double h, double inv_h) {
  const double q = dmul(d, inv_h);
  const double f = floor(q);
  const double tol = 8.8817841970012523e-16 * fabs(q);  // 8 u |q|
  if (q - f <= tol || dsub(f + 1.0, q) <= tol) return floor(d / h);
  return f;
}

// One axis of the reference cell from the FP32 mirror xf of x when that is
// provably the FP64 answer. With A = (|xf| + |bf|)/h, the FP32 quotient
// (xf - bf)(1/h) lies within 2^-24 A + 3 2^-24 |q| of the FP64 one (rounding
// of x, b, 1/h, the difference and the product); when no integer lies within
// 2^-21 (A + |q| + 1) of it, both floors agree. Otherwise (and for NaN, inf or
// |q| >= 2^22) the exact FP64 path decides.
__device__ __forceinline__ int32_t ref_axis_fast(double x, float xf, double b, float bf, double h, double inv_h,
                                                 float inv_hf) {
  const float q = (xf - bf) * inv_hf;
  const float f = floorf(q);
  const float tol = 4.76837158203125e-7f * ((fabsf(xf) + fabsf(bf)) * inv_hf + fabsf(q) + 1.0f);
  if (q - f > tol && (f + 1.0f) - q > tol) return (int32_t)f;
  return sat_i32(floor_div_exact(dsub(x, b), h, inv_h));
}

// Reference cell coordinates of a position (src/grid.rs:30-32).
__device__ __forceinline__ void ref_coords(const StepParams& P, double x, double y, double z, int32_t c[3]) {
  c[0] = sat_i32(floor_div_exact(dsub(x, P.bmin[0]), P.href, P.inv_href));
  c[1] = sat_i32(floor_div_exact(dsub(y, P.bmin[1]), P.href, P.inv_href));
  c[2] = sat_i32(floor_div_exact(dsub(z, P.bmin[2]), P.href, P.inv_href));
}

// Number of times the reference's 27-cell loop (src/grid.rs:54-85) lists the
// cell of a particle with coordinates cj when centred on ci; 0 when cj is
// outside the grid (the particle was never inserted, src/grid.rs:34-37).
__device__ __forceinline__ int ref_visits(const StepParams& P, unsigned long long ci, unsigned long long cj) {
  int m = 1;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int32_t a = code_axis(ci, k), b = code_axis(cj, k), D = P.rdims[k];
    if (b < 0 || b >= D) return 0;
    int mk = 0;
#pragma unroll
    for (int d = -1; d <= 1; ++d) {
      int32_t q = a + d;
      if (P.periodic[k]) {
        if (q < 0) q += D;
        else if (q >= D) q -= D;
      }
      mk += (q == b) ? 1 : 0;
    }
    m *= mk;
    if (m == 0) return 0;
  }
  return m;
}

// Whether a reference-cell code lies inside the grid (the reference inserted
// the particle, src/grid.rs:34-37).
__device__ __forceinline__ bool ref_inside(const StepParams& P, unsigned long long c) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int32_t b = code_axis(c, k);
    if (b < 0 || b >= P.rdims[k]) return false;
  }
  return true;
}

// Fine-grid cell of a position: periodic axes wrap, open axes clamp. The
// quotients are products with the reciprocals (a few ulps off the exact
// ones); the cells are larger than the list radius by a relative 1e-7, so two
// particles within the list radius still land in neighbouring cells.
__device__ __forceinline__ uint32_t fine_cell(const StepParams& P, double x, double y, double z) {
  double p[3] = {x, y, z};
  int c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double q = p[k] - P.fmin[k];
    if (P.periodic[k]) {
      double L = P.bsize[k];
      q = q - floor(q * P.binv[k]) * L;
    }
    double f = floor(q * P.finv[k]);
    int ck = (f != f) ? 0 : (f < 0.0 ? 0 : (f >= (double)P.fdims[k] ? P.fdims[k] - 1 : (int)f));
    c[k] = ck;
  }
  return (uint32_t)c[0] + (uint32_t)P.fdims[0] * ((uint32_t)c[1] + (uint32_t)P.fdims[1] * (uint32_t)c[2]);
}

}  // namespace rp
