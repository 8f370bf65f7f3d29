// Host engine: particle store, device buffers and step sequencing.
//
// A step is launched as: first half (the previous step's second half kick,
// boundary, kick, drift) -> gated rebuild chain (hash, radix sort, cell
// bounds, reorder, Verlet lists) -> forces (a, tau only) -> end-of-step
// bookkeeping; a stepping call ends with the pending second half kick, so the
// state between calls is the reference's end-of-step state. Steps are issued in chunks with one
// host synchronisation per chunk; a device control block reports completed
// steps, rebuilds, removals and a halt when a neighbour list outgrew its
// capacity (the engine then grows the lists and resumes the halted step).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>

#include "engine.h"

namespace rp {

void set_error(const char* fmt, ...);

#define CK(x)                                                                 \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      set_error("%s failed: %s", #x, cudaGetErrorString(e_));                 \
      return RP_E_CUDA;                                                       \
    }                                                                         \
  } while (0)

#define TRY(x)               \
  do {                       \
    int r_ = (x);            \
    if (r_ != RP_OK) return r_; \
  } while (0)

static const double kPiH = 3.14159265358979323846;

// src/material.rs:33-37 (same operation order as the oracle)
static double eff_youngs(double e1, double nu1, double e2, double nu2) {
  double inv = (1.0 - nu1 * nu1) / e1 + (1.0 - nu2 * nu2) / e2;
  return 1.0 / inv;
}
static double shear_mod(double e, double nu) { return e / (2.0 * (1.0 + nu)); }
static double physical_shear(double e1, double nu1, double e2, double nu2) {
  double g1 = shear_mod(e1, nu1), g2 = shear_mod(e2, nu2);
  return 1.0 / ((2.0 - nu1) / g1 + (2.0 - nu2) / g2);
}
// Law constants of one particle material against the wall material
// (src/material.rs:33-50, src/physics.rs:112-116, 165).
Law Engine::make_law(const Material& m) const {
  Law L;
  std::memset(&L, 0, sizeof(L));
  L.es_pp = eff_youngs(m.E, m.nu, m.E, m.nu);
  L.es_pw = eff_youngs(m.E, m.nu, wm.E, wm.nu);
  L.gs_pp = mode == RP_MODE_PARITY ? 0.0 : physical_shear(m.E, m.nu, m.E, m.nu);
  L.gamma_pp = (m.gamma + m.gamma) * 0.5;
  L.gamma_pw = (m.gamma + wm.gamma) * 0.5;
  const double ln_e = std::log(m.e);
  const double beta = ln_e / std::sqrt(ln_e * ln_e + kPiH * kPiH);
  L.beta_abs = std::fabs(beta);
  L.mu = m.mu;
  L.jkr_C = (8.0 * kPiH) * L.gamma_pp / L.es_pp;
  L.jkr_Cf = (float)L.jkr_C;
  return L;
}

static int bits_for(uint64_t maxkey) {
  int b = 1;
  while (b < 32 && (1ull << b) <= maxkey) ++b;
  return b;
}
template <typename T>
static int dalloc(T** p, size_t count) {
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    *p = nullptr;
    set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
    return RP_E_NOMEM;
  }
  return RP_OK;
}
template <typename T>
static void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

Engine::Engine(double dt_, const double mn[3], const double mx[3], size_t capacity) : dt(dt_) {
  for (int k = 0; k < 3; ++k) {
    bmin[k] = mn[k];
    bmax[k] = mx[k];
  }
  hp_.reserve(capacity);
}

Engine::~Engine() { free_device(); }

void Engine::free_device() {
  if (!gpu_) return;
  cudaSetDevice(device_);
  destroy_graph();
  if (cap_stream_) cudaStreamDestroy(cap_stream_);
  if (cap_stream2_) cudaStreamDestroy(cap_stream2_);
  cap_stream_ = cap_stream2_ = nullptr;
  for (int b = 0; b < 2; ++b) {
    Bank& B = bank_[b];
    dfree(B.xr); dfree(B.vm); dfree(B.wc); dfree(B.acc); dfree(B.tq);
    dfree(B.xres); dfree(B.vres); dfree(B.wres); dfree(B.flags); dfree(B.tag); dfree(B.xref); dfree(B.xf);
    dfree(B.grp); dfree(B.hmask);
    dfree(B.nbr); dfree(B.ncnt); dfree(B.hist);
  }
  dfree(rb_.ka); dfree(rb_.va); dfree(rb_.kb); dfree(rb_.vb); dfree(rb_.hist); dfree(rb_.part);
  dfree(rb_.cstart); dfree(rb_.cend); dfree(kraw_);
  dfree(dbgF_); dfree(dbgT_); dfree(dbgMult_); dfree(ke_);
  dfree(crec_); dfree(clist_); dfree(cres_); dfree(ccnt_); dfree(aorder_); dfree(coff_);
  dfree(warena_); dfree(wres_); dfree(wok_); dfree(woff_); dfree(wcnt_);
  dfree(ctot_);
  dfree(tri_d_); dfree(tstart_d_); dfree(titems_d_); dfree(glaw_d_); dfree(motions_d_);
  dfree(mlp_d_); dfree(jq_); dfree(jguess_); dfree(jfb_);
  dfree(io_buf_); dfree(slot_of_); dfree(io_flag_); dfree(id_live_); dfree(id_pos_); dfree(slot_of_id_);
  dfree(id_part_);
  io_n_ = 0;
  jq_alloc_ = 0;
  jfb_alloc_ = 0;
  dfree(ctrl_);
  if (ctrl_h_) cudaFreeHost(ctrl_h_);
  ctrl_h_ = nullptr;
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  for (cudaEvent_t e : fev_) cudaEventDestroy(e);
  fev_.clear();
  if (stream_) cudaStreamDestroy(stream_);
  stream_ = nullptr;
  ev0_ = ev1_ = nullptr;
  gpu_ = false;
}

void Engine::free_lists() {
  if (!gpu_) return;
  for (int b = 0; b < 2; ++b) {
    dfree(bank_[b].nbr);
    dfree(bank_[b].hist);
  }
  dfree(dbgMult_);
}

int Engine::ensure_gpu() {
  if (gpu_) {
    CK(cudaSetDevice(device_));
    return RP_OK;
  }
  int cnt = 0;
  cudaError_t e = cudaGetDeviceCount(&cnt);
  if (e != cudaSuccess || cnt == 0) {
    set_error("no usable CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0");
    return RP_E_CUDA;
  }
  if (device_ < 0) CK(cudaGetDevice(&device_));
  if (device_ >= cnt) {
    set_error("CUDA device %d does not exist (%d present)", device_, cnt);
    return RP_E_CUDA;
  }
  CK(cudaSetDevice(device_));
  CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ev0_));
  CK(cudaEventCreate(&ev1_));
  TRY(dalloc(&ctrl_, 1));
  CK(cudaMallocHost((void**)&ctrl_h_, sizeof(Ctrl)));
  TRY(dalloc(&ke_, 1));
  {
    // kernels may dereference the caller's pageable arrays when the device
    // reaches host memory coherently through the host's page tables
    int pageable = 0, host_tables = 0;
    CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device_));
    CK(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device_));
    // Staged copies by default: into and out of resident pageable pages they
    // ran at ~150 GB/s on GB300 with a steady time, while kernels on the
    // caller's arrays took 1-20 ms for the same bytes from run to run (device
    // walks of the host page tables). RP_DIRECT_STATE_IO=1 selects the kernels.
    const char* direct = std::getenv("RP_DIRECT_STATE_IO");
    io_direct_ = pageable == 1 && host_tables == 1 && direct && direct[0] == '1';
  }
  gpu_ = true;
  return RP_OK;
}

int Engine::enable_gpu(int device) {
  if (gpu_ && device >= 0 && device != device_) {
    if (!host_valid_) TRY(download());
    free_device();
    dev_valid_ = false;
  }
  if (!gpu_ && device >= 0) device_ = device;
  TRY(ensure_gpu());
  if (!dev_valid_) {
    if (!host_valid_) TRY(download());
    TRY(upload());
  }
  return RP_OK;
}

int Engine::add_particle(const double x[3], double r, double m, int fixed) {
  if (!host_valid_) TRY(download());
  HostParticle p;
  std::memset(&p, 0, sizeof(p));
  for (int k = 0; k < 3; ++k) p.x[k] = x[k];
  p.r = r;
  p.m = m;
  p.fixed = fixed ? 1 : 0;
  p.tag = next_tag_++;
  hp_.push_back(p);
  dev_valid_ = false;
  return RP_OK;
}

int Engine::add_triangles(size_t n, const float* v, const float* nrm, uint32_t group, const WallMotion* motion) {
  uint32_t mid = NO_MOTION;
  if (motion && n > 0) {
    motions_.push_back(*motion);
    mid = (uint32_t)(motions_.size() - 1);
  }
  for (size_t t = 0; t < n; ++t) {
    const float* q = v + 9 * t;
    tri_group_.push_back(group);
    tri_motion_.push_back(mid);
    for (int k = 0; k < 9; ++k) tri_v_.push_back(q[k]);
    if (nrm) {
      for (int k = 0; k < 3; ++k) tri_n_.push_back(nrm[3 * t + k]);
    } else {
      double e0[3] = {(double)q[3] - q[0], (double)q[4] - q[1], (double)q[5] - q[2]};
      double e1[3] = {(double)q[6] - q[0], (double)q[7] - q[1], (double)q[8] - q[2]};
      double c[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
      double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      for (int k = 0; k < 3; ++k) tri_n_.push_back(l > 0 ? (float)(c[k] / l) : 0.f);
    }
  }
  dev_valid_ = false;
  return RP_OK;
}

int Engine::set_particle_groups(size_t n, const uint32_t* groups) {
  if (!host_valid_) TRY(download());
  if (n != hp_.size()) {
    set_error("group array has %zu entries for %zu particles", n, hp_.size());
    return RP_E_INVALID_ARG;
  }
  for (size_t i = 0; i < n; ++i) {
    if (groups[i] >= (1u << 24)) {
      set_error("group id %u too large (at most 2^24 - 1)", groups[i]);
      return RP_E_INVALID_ARG;
    }
  }
  for (size_t i = 0; i < n; ++i) hp_[i].group = groups[i];
  dev_valid_ = false;
  return RP_OK;
}

int Engine::get_particle_groups(size_t n, uint32_t* groups) {
  if (!host_valid_) TRY(download());
  if (n != hp_.size()) {
    set_error("group array has %zu entries for %zu particles", n, hp_.size());
    return RP_E_INVALID_ARG;
  }
  for (size_t i = 0; i < n; ++i) groups[i] = hp_[i].group;
  return RP_OK;
}

int Engine::set_group_material(uint32_t group, const Material& m) {
  if (group >= (1u << 24)) {
    set_error("group id %u too large (at most 2^24 - 1)", group);
    return RP_E_INVALID_ARG;
  }
  if (group == 0) {
    pm = m;
  } else {
    if (gmat_.size() <= group) {
      gmat_.resize(group + 1, pm);
      gmat_set_.resize(group + 1, 0);
    }
    gmat_[group] = m;
    gmat_set_[group] = 1;
  }
  dev_valid_ = false;
  return RP_OK;
}

size_t Engine::count() {
  if (!host_valid_ && gpu_ && dev_valid_) {
    // live slots, without bringing the state to the host
    if (cudaSetDevice(device_) != cudaSuccess || sync_ctrl() != RP_OK) return 0;
    return (size_t)n_ - (size_t)ctrl_h_->removed;
  }
  if (!host_valid_) {
    if (download() != RP_OK) return 0;
  }
  return hp_.size();
}

// ------------------------------------------------------------- allocation
int Engine::alloc_slots(size_t n) {
  size_t na = std::max<size_t>(n, 1);
  na = (na + 1023) & ~size_t(1023);
  for (int b = 0; b < 2; ++b) {
    Bank& B = bank_[b];
    TRY(dalloc(&B.xr, na)); TRY(dalloc(&B.vm, na)); TRY(dalloc(&B.wc, na)); TRY(dalloc(&B.acc, na));
    TRY(dalloc(&B.tq, na)); TRY(dalloc(&B.xres, na)); TRY(dalloc(&B.vres, na)); TRY(dalloc(&B.wres, na));
    TRY(dalloc(&B.flags, na)); TRY(dalloc(&B.tag, na)); TRY(dalloc(&B.xref, na)); TRY(dalloc(&B.ncnt, na));
    TRY(dalloc(&B.xf, na)); TRY(dalloc(&B.grp, na)); TRY(dalloc(&B.hmask, na));
  }
  TRY(dalloc(&rb_.ka, na)); TRY(dalloc(&rb_.va, na)); TRY(dalloc(&rb_.kb, na)); TRY(dalloc(&rb_.vb, na));
  TRY(dalloc(&kraw_, na));
  uint32_t hn = radix_hist_needed((uint32_t)na);
  TRY(dalloc(&rb_.hist, hn));
  TRY(dalloc(&rb_.part, scan_parts_needed(std::max<uint32_t>(hn, (uint32_t)na)) + 16));
  TRY(dalloc(&dbgF_, 3 * na)); TRY(dalloc(&dbgT_, 3 * na));
  TRY(dalloc(&aorder_, na));
  TRY(dalloc(&woff_, na)); TRY(dalloc(&wcnt_, na));
  TRY(alloc_walls(std::max(wcap_, na / 2 + 65536)));
  TRY(dalloc(&ccnt_, na)); TRY(dalloc(&coff_, na));
  TRY(dalloc(&ctot_, 8));
  CK(cudaMemset(ctot_, 0, 8 * sizeof(uint32_t)));
  n_alloc_ = na;
  // lists must be re-allocated for the new slot count
  for (int b = 0; b < 2; ++b) {
    dfree(bank_[b].nbr);
    dfree(bank_[b].hist);
  }
  dfree(dbgMult_);
  return RP_OK;
}

// The wall candidate arena of the force pass (candidates, their results and
// contact flags), room for `cap` candidates. A filter that finds it full
// halts the step (HALT_WALLS) and recover_halt grows it.
int Engine::alloc_walls(size_t cap) {
  TRY(dalloc(&warena_, cap));
  TRY(dalloc(&wres_, 6 * cap));
  TRY(dalloc(&wok_, cap));
  wcap_ = cap;
  refresh_list_ptrs();
  return RP_OK;
}

int Engine::alloc_lists(int cap, bool keep_current) {
  const bool need_hist = (mode == RP_MODE_PHYSICAL && tmodel != RP_TANGENTIAL_COULOMB);
  const size_t na = n_alloc_;
  const int cur = keep_current ? last_.bank : 0;
  uint32_t* old_nbr = keep_current ? bank_[cur].nbr : nullptr;
  double* old_hist = keep_current ? bank_[cur].hist : nullptr;
  const int old_cap = cap_;
  for (int b = 0; b < 2; ++b) {
    uint32_t* nb = nullptr;
    TRY(dalloc(&nb, na * (size_t)cap));
    double* nh = nullptr;
    if (need_hist) {
      TRY(dalloc(&nh, 3 * na * (size_t)cap));
      CK(cudaMemsetAsync(nh, 0, sizeof(double) * 3 * na * (size_t)cap, stream_));
    }
    if (keep_current && b == cur && old_nbr && n_ > 0) {
      CK(cudaMemcpy2DAsync(nb, sizeof(uint32_t) * cap, old_nbr, sizeof(uint32_t) * old_cap,
                           sizeof(uint32_t) * old_cap, n_, cudaMemcpyDeviceToDevice, stream_));
      if (need_hist && old_hist) {
        for (int p = 0; p < 3; ++p)
          CK(cudaMemcpy2DAsync(nh + (size_t)p * n_ * cap, sizeof(double) * cap, old_hist + (size_t)p * n_ * old_cap,
                               sizeof(double) * old_cap, sizeof(double) * old_cap, n_, cudaMemcpyDeviceToDevice,
                               stream_));
      }
    }
    CK(cudaStreamSynchronize(stream_));
    dfree(bank_[b].nbr);
    dfree(bank_[b].hist);
    bank_[b].nbr = nb;
    bank_[b].hist = nh;
  }
  if (debug) {
    TRY(dalloc(&dbgMult_, na * (size_t)cap));
    CK(cudaMemset(dbgMult_, 0, na * (size_t)cap));
  } else {
    dfree(dbgMult_);
  }
  TRY(dalloc(&crec_, na * (size_t)cap));
  TRY(dalloc(&clist_, na * (size_t)cap));
  TRY(dalloc(&cres_, 6 * na * (size_t)cap));
  cap_ = cap;
  graph_dirty_ = true;
  refresh_list_ptrs();
  TRY(ensure_jkr_buffers());
  return RP_OK;
}

// Network queue and per-record predictions (one entry per possible
// evaluating record) and the device copy of the network, for the learned
// JKR solver only.
int Engine::ensure_jkr_buffers() {
  // pairs left to the reference's Newton by the certified solvers
  const bool defer = gpu_ && jkr_solver != RP_JKR_NEWTON && nmodel == RP_NORMAL_JKR;
  if (defer) {
    const size_t need = std::max<size_t>(n_alloc_ * (size_t)std::max(cap_, 1), 1);
    if (jfb_alloc_ < need) {
      TRY(dalloc(&jfb_, need));
      jfb_alloc_ = need;
      graph_dirty_ = true;
    }
    P_.jfb = jfb_;
  } else {
    P_.jfb = nullptr;
  }
  if (jkr_solver != RP_JKR_LEARNED || !gpu_ || !jkr_have_net_) {
    P_.mlp = nullptr;
    return RP_OK;
  }
  const size_t need = std::max<size_t>(n_alloc_ * (size_t)std::max(cap_, 1), 1);
  if (jq_alloc_ < need) {
    TRY(dalloc(&jq_, need));
    TRY(dalloc(&jguess_, need));
    jq_alloc_ = need;
    graph_dirty_ = true;
  }
  if (!mlp_d_) {
    TRY(dalloc(&mlp_d_, 1));
    MlpInfer h;
    mlp_make_infer(jkr_params_.data(), jkr_norm_, &h);
    CK(cudaMemcpy(mlp_d_, &h, sizeof(MlpInfer), cudaMemcpyHostToDevice));
  }
  P_.mlp = mlp_d_;
  P_.jq = jq_;
  P_.jguess = jguess_;
  return RP_OK;
}

void Engine::refresh_list_ptrs() {
  P_.cap = cap_;
  P_.bank[0] = bank_[0];
  P_.bank[1] = bank_[1];
  P_.dbgMult = dbgMult_;
  P_.crec = crec_;
  P_.clist = clist_;
  P_.cres = cres_;
  P_.cresf = reinterpret_cast<float*>(cres_);
  P_.ccnt = ccnt_;
  P_.aorder = aorder_;
  P_.warena = warena_;
  P_.wres = wres_;
  P_.wok = wok_;
  P_.woff = woff_;
  P_.wcnt = wcnt_;
  P_.wcap = (uint32_t)wcap_;
  P_.coff = coff_;
  P_.ctot = ctot_;
}

// ------------------------------------------------------------ parameters
int Engine::build_params() {
  StepParams& P = P_;
  P.n = n_;
  P.cap = cap_;
  P.nmodel = nmodel;
  P.tmodel = tmodel;
  P.mode = mode;
  P.prec = prec;
  P.debug = debug;
  P.dt = dt;
  for (int k = 0; k < 3; ++k) {
    P.periodic[k] = periodic[k] ? 1 : 0;
    P.bmin[k] = bmin[k];
    P.bmax[k] = bmax[k];
    P.bsize[k] = bmax[k] - bmin[k];
    P.bsizef[k] = (float)P.bsize[k];
    {
      const double q = 0.25 * P.bsize[k];
      uint64_t b;
      std::memcpy(&b, &q, sizeof(b));
      P.bq_hi[k] = (uint32_t)(b >> 32) & 0x7FFFFFFFu;
    }
    P.gravity[k] = gravity[k];
  }
  {
    // the FP32 mirror of a position is within 2^-24 |x| of it: a margin of
    // 1e-6 (|bounds| + 2) keeps the inner intervals inside the exact ones
    double bmag = 0.0;
    for (int k = 0; k < 3; ++k) bmag = std::max(bmag, std::max(std::fabs(bmin[k]), std::fabs(bmax[k])));
    const double m = 1e-6 * (bmag + 2.0);
    for (int k = 0; k < 3; ++k) {
      const double lo = periodic[k] ? bmin[k] + m : bmin[k] - 1.0 + m;
      const double hi = periodic[k] ? bmax[k] - m : (k == 1 ? INFINITY : bmax[k] + 1.0 - m);
      P.inner_lo[k] = std::nextafter((float)lo, INFINITY);
      P.inner_hi[k] = std::isinf(hi) ? INFINITY : std::nextafter((float)hi, -INFINITY);
    }
  }
  P.pm = pm;
  P.wm = wm;
  // per-group law constants (group 0: the particle material)
  {
    uint32_t ng = 1;
    for (const HostParticle& p : hp_) ng = std::max(ng, p.group + 1);
    for (uint32_t g : tri_group_)
      if (g != GROUP_ALL) ng = std::max(ng, g + 1);
    std::vector<Law> laws(ng);
    for (uint32_t g = 0; g < ng; ++g) {
      const Material& m = (g > 0 && g < gmat_.size() && gmat_set_[g]) ? gmat_[g] : pm;
      laws[g] = make_law(m);
    }
    P.law = laws[0];
    P.ngroups = (int)ng;
    TRY(dalloc(&glaw_d_, ng));
    CK(cudaMemcpy(glaw_d_, laws.data(), sizeof(Law) * ng, cudaMemcpyHostToDevice));
    P.glaw = glaw_d_;
  }
  // reference grid: dims = ceil(size / h) + 1 (src/grid.rs:13)
  P.href = href;
  P.inv_href = 1.0 / href;
  for (int k = 0; k < 3; ++k) {
    double q = std::ceil(P.bsize[k] / href);
    if (!(q >= 0.0) || q > (double)((1 << 20) - 4)) {
      if (mode == RP_MODE_PARITY) {
        set_error("reference grid too large on axis %d (%g cells); parity mode needs < 2^20 cells per axis", k, q);
        return RP_E_INVALID_ARG;
      }
      q = 1.0;
    }
    P.rdims[k] = (int)q + 1;
  }
  // two particles in the same inserted reference cell: each axis lists that
  // cell once, or three times on a periodic axis of a single cell (the -1, 0
  // and +1 offsets all wrap onto it), src/grid.rs:54-85
  P.same_cell_visits = 1;
  for (int k = 0; k < 3; ++k)
    if (periodic[k] && P.rdims[k] == 1) P.same_cell_visits *= 3;
  double rmax = 0.0;
  for (const HostParticle& p : hp_) rmax = std::max(rmax, p.r);
  const double adh = (nmodel == RP_NORMAL_JKR || nmodel == RP_NORMAL_SJKR) ? 1.5 : 1.0;
  double skin = skin_user > 0.0 ? skin_user : 0.1 * 2.0 * rmax;
  if (!(skin > 0.0)) skin = 1e-6;
  P.skin = skin;
  P.list_scale = 1.0f + 1e-5f;
  {
    double cutmax = 2.0 * rmax * adh;
    double lm = 0.0;
    bool ok = true;
    for (int k = 0; k < 3; ++k)
      if (periodic[k]) {
        lm = std::max(lm, P.bsize[k]);
        if (P.bsize[k] < 4.0 * cutmax) ok = false;
      }
    P.pretest = ok ? 1 : 0;
    P.lmax = (float)lm;
  }
  // fine cells at least the largest list radius, with a relative 1e-7 to
  // spare for the rounding of the cell lookup (fine_cell)
  double h = (2.0 * rmax * adh + skin) * (1.0 + 1e-7);
  if (!(h > 0.0)) h = 1.0;
  const uint64_t max_cells = std::max<uint64_t>(4ull * (uint64_t)n_ + (1ull << 16), 1ull << 20);
  for (int iter = 0; iter < 64; ++iter) {
    uint64_t tot = 1;
    for (int k = 0; k < 3; ++k) {
      double L = P.bsize[k];
      double d = periodic[k] ? std::floor(L / h) : std::ceil(L / h);
      if (!(d >= 1.0)) d = 1.0;
      if (d > 1e6) d = 1e6;
      P.fdims[k] = (int)d;
      P.fcell[k] = periodic[k] ? L / d : h;
      if (!(P.fcell[k] >= h)) P.fcell[k] = h;
      P.fmin[k] = bmin[k];
      tot *= (uint64_t)P.fdims[k];
    }
    if (tot <= max_cells) break;
    h *= 1.25;
  }
  double xb = 0.0;
  for (int k = 0; k < 3; ++k) {
    P.finv[k] = 1.0 / P.fcell[k];
    P.binv[k] = P.bsize[k] > 0.0 ? 1.0 / P.bsize[k] : 0.0;
    P.fcellf[k] = (float)P.fcell[k];
    P.binvf[k] = (float)P.binv[k];
    // live particles lie within 1.0 of the box (src/simulation.rs:199-219)
    xb = std::max(xb, std::max(std::fabs(bmin[k]), std::fabs(bmax[k])) + 1.0);
  }
  P.rmaxf = (float)rmax;
  P.xbound = (float)xb;
  P.fncells = (uint32_t)((uint64_t)P.fdims[0] * P.fdims[1] * P.fdims[2]);
  rb_.key_bits = bits_for(P.fncells);
  rb_.carry_history = (mode == RP_MODE_PHYSICAL && tmodel != RP_TANGENTIAL_COULOMB) ? 1 : 0;
  if (P.fncells > fcells_alloc_) {
    TRY(dalloc(&rb_.cstart, P.fncells));
    TRY(dalloc(&rb_.cend, P.fncells));
    fcells_alloc_ = P.fncells;
  }
  TRY(build_triangle_grid(rmax));
  P.dbgF = dbgF_;
  P.dbgT = dbgT_;
  P.ctrl = ctrl_;
  P.force_path = force_path;
  P.bs_filter = bs_filter;
  P.bs_force = bs_force;
  P.bs_accum = bs_accum;
  P.grid_cap = grid_cap;
  P.nsm = sm_count();
  P.jkr_solver = jkr_solver;
  for (int k = 0; k < 4; ++k) {
    P.jdom_lo[k] = jkr_dom_[k];
    P.jdom_hi[k] = jkr_dom_[4 + k];
  }
  refresh_list_ptrs();
  TRY(ensure_jkr_buffers());
  return RP_OK;
}

// Uniform grid over the triangles: each triangle is listed in every cell its
// bounding box, grown by the largest particle radius, overlaps and whose
// centre lies within reach of it; a particle then tests only the triangles of
// the cell holding its centre. Lists keep triangle (mesh) order, so
// contributions sum in the reference's order (src/simulation.rs:465-466).
// The host does the O(T) set-up from the mesh it holds (grown boxes, cell
// size, candidate counts); k_trigrid.cu builds the records and the lists on
// the device.
int Engine::build_triangle_grid(double rmax) {
  const size_t T = tri_v_.size() / 9;
  P_.ntri = (int)T;
  P_.motions = nullptr;
  if (T == 0) {
    P_.tri = nullptr;
    P_.tstart = nullptr;
    P_.titems = nullptr;
    P_.wall_far_ok = 0;
    return RP_OK;
  }
  if (T > (size_t)0x3FFFFFF) {
    set_error("too many triangles (%zu)", T);
    return RP_E_INVALID_ARG;
  }
  if (!motions_.empty()) {
    TRY(dalloc(&motions_d_, motions_.size()));
    CK(cudaMemcpy(motions_d_, motions_.data(), sizeof(WallMotion) * motions_.size(), cudaMemcpyHostToDevice));
    P_.motions = motions_d_;
  }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  std::vector<double> blo(3 * T), bhi(3 * T);
  // Cells are looked up in FP32 on the device (error ~1e-7 of the coordinate),
  // so bounding boxes grow by the largest radius plus an absolute margin that
  // covers a lookup landing in a neighbouring cell.
  double extent_abs = 0.0;
  for (float q : tri_v_) extent_abs = std::max(extent_abs, std::fabs((double)q));
  const double grow = rmax * (1.0 + 1e-6) + 1e-6 * (1.0 + extent_abs + rmax);
  for (size_t t = 0; t < T; ++t) {
    const float* q = &tri_v_[9 * t];
    const double v0[3] = {q[0], q[1], q[2]}, v1[3] = {q[3], q[4], q[5]}, v2[3] = {q[6], q[7], q[8]};
    for (int k = 0; k < 3; ++k) {
      double mn = std::min(v0[k], std::min(v1[k], v2[k])) - grow;
      double mx = std::max(v0[k], std::max(v1[k], v2[k])) + grow;
      blo[3 * t + k] = mn;
      bhi[3 * t + k] = mx;
      lo[k] = std::min(lo[k], mn);
      hi[k] = std::max(hi[k], mx);
    }
  }
  double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  // cells of about a radius keep the per-cell lists (pruned by distance) short
  double cell = std::max(rmax, ext / 1024.0);
  if (!(cell > 0.0)) cell = 1.0;
  int dims[3] = {1, 1, 1};
  std::vector<int> box(6 * T);
  std::vector<uint32_t> coff(T + 1, 0);
  auto cell_box = [&](size_t t, int a[3], int b[3]) {
    for (int k = 0; k < 3; ++k) {
      a[k] = std::max(0, (int)std::floor((blo[3 * t + k] - lo[k]) / cell));
      b[k] = std::min(dims[k] - 1, (int)std::floor((bhi[3 * t + k] - lo[k]) / cell));
    }
  };
  for (int iter = 0; iter < 80; ++iter) {
    uint64_t tot = 1;
    for (int k = 0; k < 3; ++k) {
      dims[k] = std::max(1, (int)std::ceil((hi[k] - lo[k]) / cell));
      tot *= (uint64_t)dims[k];
    }
    if (tot > (1ull << 24)) {
      cell *= 1.5;
      continue;
    }
    uint64_t entries = 0;
    for (size_t t = 0; t < T; ++t) {
      int a[3], b[3];
      cell_box(t, a, b);
      entries += (uint64_t)(b[0] - a[0] + 1) * (uint64_t)(b[1] - a[1] + 1) * (uint64_t)(b[2] - a[2] + 1);
    }
    if (entries <= 64ull * T + (1ull << 22)) break;
    cell *= 1.5;
  }
  uint64_t total = 0;
  for (size_t t = 0; t < T; ++t) {
    int a[3], b[3];
    cell_box(t, a, b);
    for (int k = 0; k < 3; ++k) {
      box[6 * t + k] = a[k];
      box[6 * t + 3 + k] = b[k];
    }
    coff[t] = (uint32_t)total;
    total += (uint64_t)(b[0] - a[0] + 1) * (uint64_t)(b[1] - a[1] + 1) * (uint64_t)(b[2] - a[2] + 1);
    if (total > 0xFFFFFFF0ull) {
      set_error("triangle grid too large");
      return RP_E_INVALID_ARG;
    }
  }
  coff[T] = (uint32_t)total;
  TriGridShape S;
  for (int k = 0; k < 3; ++k) {
    S.lo[k] = lo[k];
    S.dims[k] = dims[k];
  }
  S.cell = cell;
  S.ncells = (uint32_t)((size_t)dims[0] * dims[1] * dims[2]);
  // a centre that rounds into a cell and lies within rmax of the triangle is
  // within half a cell diagonal plus the growth of the cell's centre
  // (degenerate triangles keep the whole box)
  const double reach = cell * std::sqrt(3.0) * 0.5 + grow;
  S.reach2 = reach * reach * (1.0 + 1e-9) + 1e-24;
  // the mesh and the set-up go to the device; records and lists are built there
  const size_t nc = S.ncells;
  const uint32_t n = (uint32_t)total;
  float *v_d = nullptr, *n_d = nullptr;
  uint32_t *g_d = nullptr, *m_d = nullptr, *coff_d = nullptr, *ka = nullptr, *va = nullptr, *kb = nullptr,
           *vb = nullptr, *hist = nullptr, *part = nullptr, *counts = nullptr;
  int* box_d = nullptr;
  int rc = RP_OK;
  auto cleanup = [&]() {
    dfree(v_d); dfree(n_d); dfree(g_d); dfree(m_d); dfree(coff_d); dfree(box_d);
    dfree(ka); dfree(va); dfree(kb); dfree(vb); dfree(hist); dfree(part); dfree(counts);
  };
  const uint32_t hn = radix_hist_needed(std::max<uint32_t>(n, 1));
  if ((rc = dalloc(&v_d, 9 * T)) || (rc = dalloc(&n_d, 3 * T)) || (rc = dalloc(&g_d, T)) || (rc = dalloc(&m_d, T)) ||
      (rc = dalloc(&coff_d, T + 1)) || (rc = dalloc(&box_d, 6 * T)) || (rc = dalloc(&ka, n)) ||
      (rc = dalloc(&va, n)) || (rc = dalloc(&kb, n)) || (rc = dalloc(&vb, n)) || (rc = dalloc(&hist, hn)) ||
      (rc = dalloc(&part, scan_parts_needed(std::max<uint32_t>(hn, (uint32_t)nc + 1)) + 16)) ||
      (rc = dalloc(&counts, nc + 1)) || (rc = dalloc(&tri_d_, T)) || (rc = dalloc(&tstart_d_, nc + 1)) ||
      (rc = dalloc(&titems_d_, std::max<size_t>(n, 1)))) {
    cleanup();
    return rc;
  }
  cudaError_t e = cudaMemcpyAsync(v_d, tri_v_.data(), sizeof(float) * 9 * T, cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess) e = cudaMemcpyAsync(n_d, tri_n_.data(), sizeof(float) * 3 * T, cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_d, tri_group_.data(), sizeof(uint32_t) * T, cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m_d, tri_motion_.data(), sizeof(uint32_t) * T, cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(coff_d, coff.data(), sizeof(uint32_t) * (T + 1), cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess) e = cudaMemcpyAsync(box_d, box.data(), sizeof(int) * 6 * T, cudaMemcpyHostToDevice, stream_);
  const uint32_t* items = nullptr;
  if (e == cudaSuccess) {
    launch_triangle_grid(v_d, n_d, g_d, m_d, (int)T, box_d, coff_d, n, S, tri_d_, ka, va, kb, vb, hist, part,
                         counts, tstart_d_, stream_, &items);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && n > 0)
    e = cudaMemcpyAsync(titems_d_, items, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  cleanup();
  if (e != cudaSuccess) {
    set_error("triangle grid build failed: %s", cudaGetErrorString(e));
    return RP_E_CUDA;
  }
  P_.tri = tri_d_;
  P_.tstart = tstart_d_;
  P_.titems = titems_d_;
  for (int k = 0; k < 3; ++k) {
    P_.tmin[k] = lo[k];
    P_.tminf[k] = (float)lo[k];
    P_.tdims[k] = dims[k];
  }
  P_.tcell = cell;
  P_.tinvf = (float)(1.0 / cell);
  // PF_WALLFAR needs a particle to stay among the 27 cells around its cell at
  // the last rebuild, i.e. half the skin (the most it moves) below a cell
  P_.wall_far_ok = (0.5 * P_.skin * 1.01 < cell) ? 1 : 0;
  double bmag = 0.0;
  for (int k = 0; k < 3; ++k) bmag = std::max(bmag, std::max(std::fabs(P_.bmin[k]), std::fabs(P_.bmax[k])));
  P_.wall_far_gap = (float)(0.5 * P_.skin * 1.01 + 1e-6 * (1.0 + bmag));
  tgrid_built_ = true;
  return RP_OK;
}

// The device-built triangle grid (for tests): dims, origin and cell size,
// the cell starts (ncells + 1) and the triangle ids in cell order.
int Engine::debug_triangle_grid(int32_t dims[3], double lo_cell[4], uint32_t* start, size_t start_cap,
                                uint32_t* items, size_t items_cap, size_t* n_start, size_t* n_items) {
  TRY(ensure_gpu());
  if (!dev_valid_) {
    if (!host_valid_) TRY(download());
    TRY(upload());
  }
  if (P_.ntri == 0) {
    *n_start = *n_items = 0;
    return RP_OK;
  }
  const size_t nc = (size_t)P_.tdims[0] * P_.tdims[1] * P_.tdims[2];
  for (int k = 0; k < 3; ++k) {
    dims[k] = P_.tdims[k];
    lo_cell[k] = P_.tmin[k];
  }
  lo_cell[3] = P_.tcell;
  *n_start = nc + 1;
  uint32_t total = 0;
  CK(cudaMemcpy(&total, tstart_d_ + nc, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  *n_items = total;
  if (start && start_cap >= nc + 1) CK(cudaMemcpy(start, tstart_d_, sizeof(uint32_t) * (nc + 1), cudaMemcpyDeviceToHost));
  if (items && items_cap >= total && total > 0)
    CK(cudaMemcpy(items, titems_d_, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost));
  return RP_OK;
}

// --------------------------------------------------------- upload/download
int Engine::upload() {
  TRY(ensure_gpu());
  for (const HostParticle& p : hp_) {
    if (!(p.r > 0.0) || !(p.m > 0.0)) {
      set_error("particle radius and mass must be positive");
      return RP_E_INVALID_ARG;
    }
  }
  const size_t n = hp_.size();
  if (n > (size_t)0x7FFFFFF0) {
    set_error("too many particles");
    return RP_E_INVALID_ARG;
  }
  n_ = (int)n;
  if (n > n_alloc_ || n_alloc_ == 0) TRY(alloc_slots(n));
  if (cap_ == 0) cap_ = 32;
  const bool need_hist = (mode == RP_MODE_PHYSICAL && tmodel != RP_TANGENTIAL_COULOMB);
  if (!bank_[0].nbr || (need_hist && !bank_[0].hist) || (debug && !dbgMult_)) TRY(alloc_lists(cap_, false));
  // pack
  const size_t na = std::max<size_t>(n, 1);
  std::vector<D4> a8[8];
  for (auto& v : a8) v.resize(na);
  std::vector<uint32_t> flags(na, 0), tags(na, 0), groups(na, 0);
  for (size_t i = 0; i < n; ++i) {
    const HostParticle& p = hp_[i];
    groups[i] = p.group;
    a8[0][i] = D4{p.x[0], p.x[1], p.x[2], p.r};
    a8[1][i] = D4{p.v[0], p.v[1], p.v[2], p.m};
    a8[2][i] = D4{p.w[0], p.w[1], p.w[2], 0.0};
    a8[3][i] = D4{p.a[0], p.a[1], p.a[2], 0.0};
    a8[4][i] = D4{p.tau[0], p.tau[1], p.tau[2], 0.0};
    a8[5][i] = D4{p.xres[0], p.xres[1], p.xres[2], 0.0};
    a8[6][i] = D4{p.vres[0], p.vres[1], p.vres[2], 1.0 / p.m};  // .w carries 1/m
    // .w carries 1 / I = 1 / (0.4 m r^2) (constant per particle; the same
    // correctly rounded division the step would do)
    a8[7][i] = D4{p.wres[0], p.wres[1], p.wres[2], 1.0 / (0.4 * p.m * p.r * p.r)};
    flags[i] = p.fixed ? PF_FIXED : 0u;
    tags[i] = (uint32_t)i;  // the device tag is the id at upload; the insertion tag stays on the host
  }
  up_tags_.resize(n);
  for (size_t i = 0; i < n; ++i) up_tags_[i] = hp_[i].tag;
  n_upload_ = (int)n;
  rmax_dev_ = 0.0;
  for (size_t i = 0; i < n; ++i) rmax_dev_ = std::max(rmax_dev_, hp_[i].r);
  ++uploads_;
  Bank& B = bank_[0];
  D4* dst[8] = {B.xr, B.vm, B.wc, B.acc, B.tq, B.xres, B.vres, B.wres};
  if (n > 0) {
    for (int q = 0; q < 8; ++q) CK(cudaMemcpy(dst[q], a8[q].data(), sizeof(D4) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.flags, flags.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.tag, tags.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.grp, groups.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    std::vector<float4> xref(n, make_float4(NAN, NAN, NAN, 0.f));
    CK(cudaMemcpy(B.xref, xref.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    for (size_t i = 0; i < n; ++i)
      xref[i] = make_float4((float)hp_[i].x[0], (float)hp_[i].x[1], (float)hp_[i].x[2], (float)hp_[i].r);
    CK(cudaMemcpy(B.xf, xref.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    std::vector<uint32_t> iota(n);  // replaced by the first list rebuild
    for (size_t i = 0; i < n; ++i) iota[i] = (uint32_t)i;
    CK(cudaMemcpy(aorder_, iota.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
  }
  for (int b = 0; b < 2; ++b) CK(cudaMemset(bank_[b].ncnt, 0, sizeof(uint32_t) * n_alloc_));
  if (need_hist)
    for (int b = 0; b < 2; ++b) {
      CK(cudaMemset(bank_[b].hist, 0, sizeof(double) * 3 * n_alloc_ * (size_t)cap_));
      CK(cudaMemset(bank_[b].hmask, 0, sizeof(unsigned long long) * n_alloc_));
    }
  TRY(build_params());
  Ctrl c;
  std::memset(&c, 0, sizeof(c));
  c.bank = 0;
  c.rebuild = 1;
  CK(cudaMemcpy(ctrl_, &c, sizeof(Ctrl), cudaMemcpyHostToDevice));
  last_ = c;
  dev_valid_ = true;
  graph_dirty_ = true;  // kernel parameters changed
  return RP_OK;
}

int Engine::sync_ctrl() {
  CK(cudaMemcpyAsync(ctrl_h_, ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  return RP_OK;
}

int Engine::download() {
  if (!gpu_ || !dev_valid_ || host_valid_) {
    host_valid_ = true;
    return RP_OK;
  }
  CK(cudaSetDevice(device_));
  TRY(sync_ctrl());
  ++downloads_;
  const Bank& B = bank_[ctrl_h_->bank];
  const size_t n = (size_t)n_;
  std::vector<D4> a8[8];
  const D4* src[8] = {B.xr, B.vm, B.wc, B.acc, B.tq, B.xres, B.vres, B.wres};
  std::vector<uint32_t> flags(n), tags(n), groups(n, 0u);
  if (n > 0) {
    for (int q = 0; q < 8; ++q) {
      a8[q].resize(n);
      CK(cudaMemcpy(a8[q].data(), src[q], sizeof(D4) * n, cudaMemcpyDeviceToHost));
    }
    CK(cudaMemcpy(flags.data(), B.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(tags.data(), B.tag, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    if (P_.ngroups > 1) CK(cudaMemcpy(groups.data(), B.grp, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
  }
  std::vector<std::pair<uint32_t, size_t>> order;
  order.reserve(n);
  bool dead = false;
  for (size_t k = 0; k < n; ++k) {
    if (flags[k] & PF_DEAD) {
      dead = true;
      continue;
    }
    order.emplace_back(tags[k], k);
  }
  std::sort(order.begin(), order.end());
  hp_.resize(order.size());
  for (size_t i = 0; i < order.size(); ++i) {
    size_t k = order[i].second;
    HostParticle& p = hp_[i];
    const D4* q[8];
    for (int a = 0; a < 8; ++a) q[a] = &a8[a][k];
    double* d[8] = {p.x, p.v, p.w, p.a, p.tau, p.xres, p.vres, p.wres};
    for (int a = 0; a < 8; ++a) {
      d[a][0] = q[a]->x;
      d[a][1] = q[a]->y;
      d[a][2] = q[a]->z;
    }
    p.r = a8[0][k].w;
    p.m = a8[1][k].w;
    p.fixed = (flags[k] & PF_FIXED) ? 1 : 0;
    p.tag = up_tags_[tags[k]];
    p.group = groups[k];
  }
  host_valid_ = true;
  if (dead) dev_valid_ = false;  // the next step re-uploads the compacted set
  return RP_OK;
}

// ------------------------------------------------------------------ steps
int Engine::finish_step_accounting() {
  const Ctrl& c = *ctrl_h_;
  tot_.steps += c.steps_done - last_.steps_done;
  tot_.rebuilds += c.rebuilds - last_.rebuilds;
  tot_.overlap_steps += c.overlap_steps - last_.overlap_steps;
  tot_.removed += c.removed - last_.removed;
  tot_.status |= c.status;
  tot_.max_count = c.max_count;
  last_ = c;
  return RP_OK;
}

// A list outgrew its capacity during the rebuild of the step after
// `steps_done`, or the wall candidates their arena during its contact filter
// (that step's first half already ran): grow the lists (keeping the current
// bank's rows for the history carry-over) or the arena, and finish that step.
int Engine::recover_halt() {
  while (ctrl_h_->halt) {
    if (ctrl_h_->halt & HALT_LISTS) {
      int newcap = std::max<int>(cap_ + 8, (int)(ctrl_h_->max_count * 5 / 4 + 8));
      TRY(alloc_lists(newcap, true));
      tot_.status |= ST_NLIST_GROW;
    }
    if (ctrl_h_->halt & HALT_WALLS) {
      TRY(alloc_walls(std::max<size_t>(wcap_ * 2, (size_t)ctrl_h_->wall_need * 5 / 4 + 65536)));
      tot_.status |= ST_WALL_GROW;
    }
    graph_dirty_ = true;
    int zero = 0;
    unsigned zu = 0;
    CK(cudaMemcpyAsync(&ctrl_->halt, &zero, sizeof(int), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(&ctrl_->max_count, &zu, sizeof(unsigned), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(&ctrl_->wall_need, &zu, sizeof(unsigned), cudaMemcpyHostToDevice, stream_));
    CK(cudaStreamSynchronize(stream_));
    launches_ += launch_rebuild(P_, rb_, stream_);
    launches_ += launch_force(P_, stream_);
    launches_ += launch_end_step(P_, stream_);
    CK(cudaGetLastError());
    TRY(sync_ctrl());
  }
  return RP_OK;
}

void Engine::destroy_graph() {
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  if (graph_) cudaGraphDestroy(graph_);
  graph_exec_ = nullptr;
  graph_ = nullptr;
}

// The device step loop: a WHILE node whose body is one step (first half,
// rebuild condition, IF node holding the rebuild chain, forces, end of
// step). k_end_step sets the loop condition from the device counters, so a
// stepping call of any length is one graph launch and the host never has to
// decide whether a step needs a rebuild.
int Engine::build_graph() {
  destroy_graph();
  if (!cap_stream_) {
    CK(cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&cap_stream2_, cudaStreamNonBlocking));
  }
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  graph_ = g;
  cudaGraphConditionalHandle hloop;
  CK(cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = hloop;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t wnode;
  CK(cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  cudaGraphConditionalHandle hif;
  CK(cudaGraphConditionalHandleCreate(&hif, body, 0, cudaGraphCondAssignDefault));
  CK(cudaStreamBeginCaptureToGraph(cap_stream_, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  int sk = launch_first_half(P_, cap_stream_);
  sk += launch_rebuild_condition(P_, hif, cap_stream_);
  cudaStreamCaptureStatus st;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(cap_stream_, &st, nullptr, &cg, &deps, nullptr, &nd));
  cudaGraphNodeParams ip = {};
  ip.type = cudaGraphNodeTypeConditional;
  ip.conditional.handle = hif;
  ip.conditional.type = cudaGraphCondTypeIf;
  ip.conditional.size = 1;
  cudaGraphNode_t inode;
  CK(cudaGraphAddNode(&inode, cg, deps, nullptr, nd, &ip));
  CK(cudaStreamUpdateCaptureDependencies(cap_stream_, &inode, nullptr, 1, cudaStreamSetCaptureDependencies));
  CK(cudaStreamBeginCaptureToGraph(cap_stream2_, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                   cudaStreamCaptureModeRelaxed));
  chain_kernels_ = launch_rebuild(P_, rb_, cap_stream2_);
  cudaGraph_t t2 = nullptr;
  CK(cudaStreamEndCapture(cap_stream2_, &t2));
  sk += launch_force(P_, cap_stream_);
  sk += launch_end_step_loop(P_, hloop, cap_stream_);
  step_kernels_ = sk;
  cudaGraph_t t1 = nullptr;
  CK(cudaStreamEndCapture(cap_stream_, &t1));
  CK(cudaGraphInstantiate(&graph_exec_, g, 0));
  graph_dirty_ = false;
  return RP_OK;
}

int Engine::launch_steps_graph(uint64_t n) {
  uint64_t remaining = n;
  while (remaining > 0) {
    // The graph bakes in the kernel parameters (buffer pointers, list
    // capacity): recover_halt reallocates the lists, so it is rebuilt before
    // every launch that follows a change.
    if (graph_dirty_ || !graph_exec_) {
      int r = build_graph();
      if (r != RP_OK) {
        // conditional graph nodes unavailable: host-issued steps instead
        destroy_graph();
        use_graph_ = false;
        cudaGetLastError();
        return launch_steps(remaining);
      }
    }
    const uint64_t before = last_.steps_done, rb_before = last_.rebuilds;
    unsigned long long lim[2] = {before + remaining, 0ull};  // target, iters
    CK(cudaMemcpyAsync(&ctrl_->target, &lim[0], sizeof(unsigned long long), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(&ctrl_->iters, &lim[1], sizeof(unsigned long long), cudaMemcpyHostToDevice, stream_));
    CK(cudaEventRecord(ev0_, stream_));
    CK(cudaGraphLaunch(graph_exec_, stream_));
    CK(cudaEventRecord(ev1_, stream_));
    TRY(sync_ctrl());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    ms_total_ += ms;
    TRY(recover_halt());
    launches_ += (uint64_t)step_kernels_ * (ctrl_h_->steps_done - before) +
                 (uint64_t)chain_kernels_ * (ctrl_h_->rebuilds - rb_before);
    TRY(finish_step_accounting());
    const uint64_t done = last_.steps_done - before;
    if (done == 0) {
      set_error("device step loop made no progress");
      return RP_E_DEVICE_FLAG;
    }
    remaining -= std::min(done, remaining);
  }
  return RP_OK;
}

// Host-issued steps in chunks (used when profiling per force launch): the
// same kernels as the device loop, every rebuild kernel gated on the device.
int Engine::launch_steps(uint64_t n) {
  const uint64_t CHUNK = 512;
  if (profiling && fev_.size() < 2 * CHUNK) {
    while (fev_.size() < 2 * CHUNK) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      fev_.push_back(e);
    }
  }
  uint64_t remaining = n;
  while (remaining > 0) {
    const uint64_t chunk = std::min(remaining, CHUNK);
    const uint64_t before = last_.steps_done;
    CK(cudaEventRecord(ev0_, stream_));
    for (uint64_t s = 0; s < chunk; ++s) {
      launches_ += launch_first_half(P_, stream_);
      launches_ += launch_rebuild(P_, rb_, stream_);
      if (profiling) CK(cudaEventRecord(fev_[2 * s], stream_));
      launches_ += launch_force(P_, stream_);
      if (profiling) CK(cudaEventRecord(fev_[2 * s + 1], stream_));
      launches_ += launch_end_step(P_, stream_);
    }
    CK(cudaEventRecord(ev1_, stream_));
    CK(cudaGetLastError());
    TRY(sync_ctrl());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    ms_total_ += ms;
    if (profiling) {
      for (uint64_t s = 0; s < chunk; ++s) {
        float fm = 0.f;
        if (cudaEventElapsedTime(&fm, fev_[2 * s], fev_[2 * s + 1]) == cudaSuccess) {
          force_ms_ += fm;
          force_launches_ += 1;
        }
      }
    }
    TRY(recover_halt());
    TRY(finish_step_accounting());
    const uint64_t done = last_.steps_done - before;
    if (done == 0) {
      set_error("device made no progress in a chunk of %llu steps", (unsigned long long)chunk);
      return RP_E_DEVICE_FLAG;
    }
    remaining -= std::min(done, remaining);
  }
  return RP_OK;
}

int Engine::step(uint64_t n) {
  TRY(ensure_gpu());
  if (!dev_valid_) {
    if (!host_valid_) TRY(download());
    TRY(upload());
  }
  if (n == 0) return RP_OK;
  if (n_ == 0) {
    tot_.steps += n;
    return RP_OK;
  }
  host_valid_ = false;
  int r = (use_graph_ && !profiling) ? launch_steps_graph(n) : launch_steps(n);
  if (r != RP_OK) return r;
  launches_ += launch_second_half(P_, stream_);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(stream_));
  if (last_.removed > 0) TRY(compact_removed());
  return RP_OK;
}

// Removed particles leave the slots on the device (src/simulation.rs:199-219
// drops them and re-indexes the rest). A rebuild of the lists sorts every
// slot by its fine-grid cell, and a dead slot's key lies past every cell, so
// after it the live slots are exactly [0, n_live): dropping the dead ones is
// setting the slot count. The ids of the live particles keep coming from the
// scan of the live flags over the upload positions (launch_slot_of), which is
// the reference's re-indexing in insertion order. The next step rebuilds the
// lists and the visiting order for the new count.
int Engine::compact_removed() {
  TRY(sync_ctrl());
  const uint64_t dead = ctrl_h_->removed;
  if (dead == 0 || ctrl_h_->halt) return RP_OK;
  for (int tries = 0;; ++tries) {
    const int one = 1;
    CK(cudaMemcpyAsync(&ctrl_->rebuild, &one, sizeof(int), cudaMemcpyHostToDevice, stream_));
    launches_ += launch_rebuild(P_, rb_, stream_);
    CK(cudaGetLastError());
    TRY(sync_ctrl());
    if (!ctrl_h_->halt) break;
    if (tries >= 8) {
      set_error("neighbour lists keep overflowing while compacting removed particles");
      return RP_E_DEVICE_FLAG;
    }
    // a list outgrew its capacity in that rebuild (the bank did not flip):
    // grow the lists and run the rebuild again from the same bank
    const int newcap = std::max<int>(cap_ + 8, (int)(ctrl_h_->max_count * 5 / 4 + 8));
    TRY(alloc_lists(newcap, true));
    tot_.status |= ST_NLIST_GROW;
    const int zero = 0;
    const unsigned zu = 0;
    CK(cudaMemcpyAsync(&ctrl_->halt, &zero, sizeof(int), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(&ctrl_->max_count, &zu, sizeof(unsigned), cudaMemcpyHostToDevice, stream_));
  }
  tot_.rebuilds += ctrl_h_->rebuilds - last_.rebuilds;
  n_ -= (int)dead;
  P_.n = n_;
  const unsigned long long zero64 = 0;
  const int one = 1;
  CK(cudaMemcpyAsync(&ctrl_->removed, &zero64, sizeof(zero64), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(&ctrl_->rebuild, &one, sizeof(int), cudaMemcpyHostToDevice, stream_));
  TRY(sync_ctrl());
  last_ = *ctrl_h_;
  graph_dirty_ = true;  // the slot count is a kernel parameter
  ++compactions_;
  return RP_OK;
}

// Insertion while the device holds the state (src/simulation.rs:93-96 pushes
// to the end of the particle list): the new particles take the slots after the
// live ones in the current bank, with upload positions after every existing
// one (so their ids follow all current ids), and the next step rebuilds the
// lists. Applies when the slots have room and the new radii do not exceed the
// largest uploaded radius (the grids are sized by it); otherwise the caller
// takes the host path (a fresh upload).
int Engine::append_on_device(size_t k, const double* xyz, const double* r, const double* m, const uint8_t* fixed,
                             bool& done) {
  done = false;
  if (!gpu_ || !dev_valid_ || k == 0 || P_.ngroups > 1) return RP_OK;
  if ((size_t)n_ + k > n_alloc_ || (size_t)n_upload_ + k > (size_t)0x7FFFFFF0) return RP_OK;
  for (size_t i = 0; i < k; ++i)
    if (!(r[i] > 0.0) || !(m[i] > 0.0) || r[i] > rmax_dev_) return RP_OK;
  CK(cudaSetDevice(device_));
  TRY(sync_ctrl());
  if (ctrl_h_->halt || ctrl_h_->pending || ctrl_h_->removed) return RP_OK;
  std::vector<D4> a8[8];
  for (auto& v : a8) v.assign(k, D4{0.0, 0.0, 0.0, 0.0});
  std::vector<uint32_t> flags(k), tags(k), zero(k, 0u);
  std::vector<float4> xf(k), xref(k, make_float4(NAN, NAN, NAN, 0.f));
  for (size_t i = 0; i < k; ++i) {
    a8[0][i] = D4{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], r[i]};
    a8[1][i] = D4{0.0, 0.0, 0.0, m[i]};
    a8[6][i] = D4{0.0, 0.0, 0.0, 1.0 / m[i]};
    a8[7][i] = D4{0.0, 0.0, 0.0, 1.0 / (0.4 * m[i] * r[i] * r[i])};
    flags[i] = (fixed && fixed[i]) ? PF_FIXED : 0u;
    tags[i] = (uint32_t)(n_upload_ + i);
    xf[i] = make_float4((float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2], (float)r[i]);
  }
  const Bank& B = bank_[ctrl_h_->bank];
  D4* dst[8] = {B.xr, B.vm, B.wc, B.acc, B.tq, B.xres, B.vres, B.wres};
  const size_t o = (size_t)n_;
  for (int q = 0; q < 8; ++q)
    CK(cudaMemcpyAsync(dst[q] + o, a8[q].data(), sizeof(D4) * k, cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(B.flags + o, flags.data(), sizeof(uint32_t) * k, cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(B.tag + o, tags.data(), sizeof(uint32_t) * k, cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(B.grp + o, zero.data(), sizeof(uint32_t) * k, cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(B.xf + o, xf.data(), sizeof(float4) * k, cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(B.xref + o, xref.data(), sizeof(float4) * k, cudaMemcpyHostToDevice, stream_));
  for (int b = 0; b < 2; ++b)
    CK(cudaMemcpyAsync(bank_[b].ncnt + o, zero.data(), sizeof(uint32_t) * k, cudaMemcpyHostToDevice, stream_));
  {  // the visiting order of the force kernels covers the new slots until the rebuild
    std::vector<uint32_t> ids(k);
    for (size_t i = 0; i < k; ++i) ids[i] = (uint32_t)(o + i);
    CK(cudaMemcpyAsync(aorder_ + o, ids.data(), sizeof(uint32_t) * k, cudaMemcpyHostToDevice, stream_));
  }
  const int one = 1;
  CK(cudaMemcpyAsync(&ctrl_->rebuild, &one, sizeof(int), cudaMemcpyHostToDevice, stream_));
  CK(cudaStreamSynchronize(stream_));
  for (size_t i = 0; i < k; ++i) {
    up_tags_.push_back(next_tag_);
    if (host_valid_) {
      HostParticle p;
      std::memset(&p, 0, sizeof(p));
      for (int a = 0; a < 3; ++a) p.x[a] = xyz[3 * i + a];
      p.r = r[i];
      p.m = m[i];
      p.fixed = (fixed && fixed[i]) ? 1 : 0;
      p.tag = next_tag_;
      hp_.push_back(p);
    }
    ++next_tag_;
  }
  n_ += (int)k;
  n_upload_ += (int)k;
  P_.n = n_;
  graph_dirty_ = true;
  device_inserts_ += k;
  done = true;
  return RP_OK;
}

int Engine::add_particles(size_t k, const double* xyz, const double* r, const double* m, const uint8_t* fixed) {
  bool done = false;
  TRY(append_on_device(k, xyz, r, m, fixed, done));
  if (done) return RP_OK;
  for (size_t i = 0; i < k; ++i) TRY(add_particle(xyz + 3 * i, r[i], m[i], fixed ? fixed[i] : 0));
  return RP_OK;
}

// ---------------------------------------------------------- state access
int Engine::get_vec(size_t id, int which, double out[3]) {
  if (!host_valid_) TRY(download());
  if (id >= hp_.size()) {
    set_error("Particle index out of bounds");
    return RP_E_INDEX;
  }
  const HostParticle& p = hp_[id];
  const double* s = which == 0 ? p.x : which == 1 ? p.v : p.w;
  for (int k = 0; k < 3; ++k) out[k] = s[k];
  return RP_OK;
}

int Engine::set_vec(size_t id, int which, const double in[3]) {
  if (!host_valid_) TRY(download());
  if (id >= hp_.size()) {
    set_error("Particle index out of bounds");
    return RP_E_INDEX;
  }
  HostParticle& p = hp_[id];
  double* d = which == 1 ? p.v : p.w;
  for (int k = 0; k < 3; ++k) d[k] = in[k];
  dev_valid_ = false;
  return RP_OK;
}

int Engine::ensure_io(size_t n) {
  if (io_buf_ && io_n_ >= n) return RP_OK;
  TRY(dalloc(&io_buf_, 26 * n + n / 8 + 1));
  TRY(dalloc(&slot_of_, n));
  TRY(dalloc(&id_live_, n));
  TRY(dalloc(&id_pos_, n));
  TRY(dalloc(&slot_of_id_, n));
  TRY(dalloc(&id_part_, scan_parts_needed((uint32_t)n) + 16));
  TRY(dalloc(&io_flag_, 1));
  io_n_ = n;
  return RP_OK;
}

// Staging layout in io_buf_: vector q at q*3n, radius at 24n, mass at 25n,
// fixed bytes at 26n.
static StateIO state_io(double* buf, size_t n, double* const vec[8], const void* r, const void* m,
                        const void* f) {
  StateIO io{};
  for (int q = 0; q < 8; ++q) io.v[q] = vec[q] ? buf + (size_t)q * 3 * n : nullptr;
  io.radius = r ? buf + 24 * n : nullptr;
  io.mass = m ? buf + 25 * n : nullptr;
  io.fixed = f ? reinterpret_cast<uint8_t*>(buf + 26 * n) : nullptr;
  return io;
}

// Writes a zero every 4 KB of each range, in parallel, so that the pages
// exist before the device writes them: a first touch of a host page from the
// device costs far more than one from the host. Every byte of the ranges is
// overwritten by the gather that follows.
static void touch_pages(const std::vector<std::pair<char*, size_t>>& ranges) {
  size_t total = 0;
  for (const auto& r : ranges) total += r.second;
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const unsigned nt = total < ((size_t)8 << 20) ? 1u : hw;
  auto work = [&](unsigned t) {
    for (const auto& r : ranges) {
      const size_t pages = (r.second + 4095) / 4096;
      for (size_t q = t; q < pages; q += nt) reinterpret_cast<volatile char*>(r.first)[q * 4096] = 0;
    }
  };
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
}

int Engine::fast_read_state(rp_state* st, bool& done) {
  done = false;
  if (!gpu_ || !dev_valid_ || n_ <= 0) return RP_OK;
  CK(cudaSetDevice(device_));
  TRY(sync_ctrl());
  if (ctrl_h_->halt != 0) return RP_OK;
  const size_t n = (size_t)n_ - (size_t)ctrl_h_->removed;  // ids of the live particles
  TRY(ensure_io((size_t)std::max(n_, n_upload_)));
  double* vec[8] = {st->position, st->velocity, st->angular_velocity, st->acceleration,
                    st->torque, st->position_residual, st->velocity_residual, st->angular_velocity_residual};
  const uint32_t* ids =
      launch_slot_of(P_, IdMap{slot_of_, id_live_, id_pos_, slot_of_id_, id_part_}, (int)n, n_upload_, stream_);
  if (io_direct_) {  // the gather writes the caller's arrays
    std::vector<std::pair<char*, size_t>> ranges;
    for (int q = 0; q < 8; ++q)
      if (vec[q]) ranges.emplace_back(reinterpret_cast<char*>(vec[q]), sizeof(double) * 3 * n);
    if (st->radius) ranges.emplace_back(reinterpret_cast<char*>(st->radius), sizeof(double) * n);
    if (st->mass) ranges.emplace_back(reinterpret_cast<char*>(st->mass), sizeof(double) * n);
    if (st->fixed) ranges.emplace_back(reinterpret_cast<char*>(st->fixed), n);
    touch_pages(ranges);
    StateIO io{};
    for (int q = 0; q < 8; ++q) io.v[q] = vec[q];
    io.radius = st->radius;
    io.mass = st->mass;
    io.fixed = st->fixed;
    launch_state_gather(P_, ids, io, (int)n, stream_);
    CK(cudaStreamSynchronize(stream_));
    CK(cudaGetLastError());
    st->n_particles = n;
    done = true;
    return RP_OK;
  }
  const StateIO io = state_io(io_buf_, n, vec, st->radius, st->mass, st->fixed);
  launch_state_gather(P_, ids, io, (int)n, stream_);
  for (int q = 0; q < 8; ++q)
    if (vec[q]) CK(cudaMemcpyAsync(vec[q], io.v[q], sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream_));
  if (st->radius) CK(cudaMemcpyAsync(st->radius, io.radius, sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
  if (st->mass) CK(cudaMemcpyAsync(st->mass, io.mass, sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
  if (st->fixed) CK(cudaMemcpyAsync(st->fixed, io.fixed, n, cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  CK(cudaGetLastError());
  st->n_particles = n;
  done = true;
  return RP_OK;
}

int Engine::fast_write_state(const rp_state* st, bool& done) {
  done = false;
  if (!gpu_ || !dev_valid_ || n_ <= 0) return RP_OK;
  CK(cudaSetDevice(device_));
  TRY(sync_ctrl());
  if (ctrl_h_->halt != 0) return RP_OK;
  const size_t n = (size_t)n_ - (size_t)ctrl_h_->removed;  // ids of the live particles
  TRY(ensure_io((size_t)std::max(n_, n_upload_)));
  double* const vec[8] = {st->position, st->velocity, st->angular_velocity, st->acceleration,
                          st->torque, st->position_residual, st->velocity_residual, st->angular_velocity_residual};
  StateIO io{};
  const uint32_t* ids =
      launch_slot_of(P_, IdMap{slot_of_, id_live_, id_pos_, slot_of_id_, id_part_}, (int)n, n_upload_, stream_);
  if (io_direct_) {  // the kernels read the caller's arrays
    for (int q = 0; q < 8; ++q) io.v[q] = vec[q];
    io.radius = st->radius;
    io.mass = st->mass;
    io.fixed = st->fixed;
  } else {
    io = state_io(io_buf_, n, vec, st->radius, st->mass, st->fixed);
    for (int q = 0; q < 8; ++q)
      if (vec[q]) CK(cudaMemcpyAsync(io.v[q], vec[q], sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream_));
    if (st->radius) CK(cudaMemcpyAsync(io.radius, st->radius, sizeof(double) * n, cudaMemcpyHostToDevice, stream_));
    if (st->mass) CK(cudaMemcpyAsync(io.mass, st->mass, sizeof(double) * n, cudaMemcpyHostToDevice, stream_));
    if (st->fixed) CK(cudaMemcpyAsync(io.fixed, st->fixed, n, cudaMemcpyHostToDevice, stream_));
  }
  if (st->radius || st->mass || st->fixed) {
    // new radii, masses or fixed flags change per-particle constants: only
    // values equal to the current ones stay on this path
    launch_state_same(P_, ids, io, io_flag_, (int)n, stream_);
    unsigned differs = 0;
    CK(cudaMemcpyAsync(&differs, io_flag_, sizeof(unsigned), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    if (differs) return RP_OK;
  }
  launch_state_scatter(P_, ids, io, (int)n, stream_);
  CK(cudaStreamSynchronize(stream_));
  CK(cudaGetLastError());
  host_valid_ = false;  // the device holds the new state
  done = true;
  return RP_OK;
}

int Engine::read_state(rp_state* st) {
  {
    bool done = false;
    TRY(fast_read_state(st, done));
    if (done) return RP_OK;
  }
  if (!host_valid_) TRY(download());
  const size_t n = hp_.size();
  st->n_particles = n;
  double* vec[8] = {st->position, st->velocity, st->angular_velocity, st->acceleration,
                    st->torque, st->position_residual, st->velocity_residual, st->angular_velocity_residual};
  for (size_t i = 0; i < n; ++i) {
    const HostParticle& p = hp_[i];
    const double* s[8] = {p.x, p.v, p.w, p.a, p.tau, p.xres, p.vres, p.wres};
    for (int a = 0; a < 8; ++a)
      if (vec[a])
        for (int k = 0; k < 3; ++k) vec[a][3 * i + k] = s[a][k];
    if (st->radius) st->radius[i] = p.r;
    if (st->mass) st->mass[i] = p.m;
    if (st->fixed) st->fixed[i] = p.fixed;
  }
  return RP_OK;
}

int Engine::write_state(const rp_state* st) {
  {
    bool done = false;
    TRY(fast_write_state(st, done));
    if (done) return RP_OK;
  }
  if (!host_valid_) TRY(download());
  const size_t n = hp_.size();
  const double* vec[8] = {st->position, st->velocity, st->angular_velocity, st->acceleration,
                          st->torque, st->position_residual, st->velocity_residual, st->angular_velocity_residual};
  for (size_t i = 0; i < n; ++i) {
    HostParticle& p = hp_[i];
    double* d[8] = {p.x, p.v, p.w, p.a, p.tau, p.xres, p.vres, p.wres};
    for (int a = 0; a < 8; ++a)
      if (vec[a])
        for (int k = 0; k < 3; ++k) d[a][k] = vec[a][3 * i + k];
    if (st->radius) p.r = st->radius[i];
    if (st->mass) p.m = st->mass[i];
    if (st->fixed) p.fixed = st->fixed[i] ? 1 : 0;
  }
  dev_valid_ = false;
  return RP_OK;
}

int Engine::stats(rp_stats* s) {
  std::memset(s, 0, sizeof(*s));
  s->steps = tot_.steps;
  s->removed = tot_.removed;
  s->neighbor_rebuilds = tot_.rebuilds;
  s->overlap_warn_steps = tot_.overlap_steps;
  s->status_bits = tot_.status;
  s->neighbor_capacity = (uint64_t)cap_;
  s->max_neighbors = tot_.max_count;
  s->device_ms = ms_total_;
  s->kernel_launches = launches_;
  s->force_launches = force_launches_;
  s->force_ms = force_ms_;
  s->state_io_direct = io_direct_ ? 1u : 0u;
  s->state_uploads = uploads_;
  s->state_downloads = downloads_;
  s->compactions = compactions_;
  s->device_inserts = device_inserts_;
  if (gpu_ && dev_valid_ && n_ > 0) {
    CK(cudaSetDevice(device_));
    launch_kinetic_energy(P_, ke_, stream_);
    double ke = 0.0;
    CK(cudaMemcpyAsync(&ke, ke_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    s->kinetic_energy = ke;
    TRY(sync_ctrl());
    s->particles = (uint64_t)n_ - (ctrl_h_->removed);
  } else {
    double ke = 0.0;
    for (const HostParticle& p : hp_) {
      double I = 0.4 * p.m * p.r * p.r;
      ke += 0.5 * p.m * (p.v[0] * p.v[0] + p.v[1] * p.v[1] + p.v[2] * p.v[2]) +
            0.5 * I * (p.w[0] * p.w[0] + p.w[1] * p.w[1] + p.w[2] * p.w[2]);
    }
    s->kinetic_energy = ke;
    s->particles = hp_.size();
  }
  return RP_OK;
}

// Bed statistics of the current state (the reference's scripts and the
// long-run statistical checks use these three): kinetic energy, coordination number (2 x
// overlapping pairs / particles) and the spheres' volume over the box's.
int Engine::bed_statistics(double out[3]) {
  TRY(ensure_gpu());
  if (!dev_valid_ || last_.steps_done == 0) {
    set_error("step at least once before asking for bed statistics (the count runs over the neighbour lists)");
    return RP_E_INVALID_ARG;
  }
  CK(cudaSetDevice(device_));
  TRY(sync_ctrl());
  double* d = nullptr;
  TRY(dalloc(&d, 3));
  launch_bed_stats(P_, d, reinterpret_cast<unsigned long long*>(d + 2), stream_);
  double h[3] = {0.0, 0.0, 0.0};
  cudaError_t e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  dfree(d);
  if (e != cudaSuccess) {
    set_error("bed statistics failed: %s", cudaGetErrorString(e));
    return RP_E_CUDA;
  }
  unsigned long long pairs = 0;
  std::memcpy(&pairs, &h[2], sizeof(pairs));
  const double n = (double)n_ - (double)ctrl_h_->removed;
  const double vbox = (bmax[0] - bmin[0]) * (bmax[1] - bmin[1]) * (bmax[2] - bmin[2]);
  out[0] = h[0];
  out[1] = n > 0.0 ? (double)pairs / n : 0.0;
  out[2] = vbox > 0.0 ? h[1] / vbox : 0.0;
  return RP_OK;
}

// ------------------------------------------------------------ diagnostics
int Engine::debug_forces(double* F, double* T) {
  if (!gpu_ || !debug) {
    set_error("debug recording is off (call rp_set_debug before stepping)");
    return RP_E_INVALID_ARG;
  }
  TRY(sync_ctrl());
  const Bank& B = bank_[ctrl_h_->bank];
  const size_t n = (size_t)n_;
  std::vector<uint32_t> flags(n), tags(n);
  std::vector<double> f(3 * n), t(3 * n);
  if (n) {
    CK(cudaMemcpy(flags.data(), B.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(tags.data(), B.tag, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(f.data(), dbgF_, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(t.data(), dbgT_, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost));
  }
  std::vector<std::pair<uint32_t, size_t>> order;
  for (size_t k = 0; k < n; ++k)
    if (!(flags[k] & PF_DEAD)) order.emplace_back(tags[k], k);
  std::sort(order.begin(), order.end());
  for (size_t i = 0; i < order.size(); ++i) {
    size_t k = order[i].second;
    for (int a = 0; a < 3; ++a) {
      F[3 * i + a] = f[3 * k + a];
      T[3 * i + a] = t[3 * k + a];
    }
  }
  return RP_OK;
}

int Engine::debug_pairs(int64_t* pi, int64_t* pj, int32_t* visits, size_t capacity, size_t* nout) {
  if (!gpu_ || !debug || !dbgMult_) {
    set_error("debug recording is off (call rp_set_debug before stepping)");
    return RP_E_INVALID_ARG;
  }
  TRY(sync_ctrl());
  const Bank& B = bank_[ctrl_h_->bank];
  const size_t n = (size_t)n_;
  std::vector<uint32_t> flags(n), tags(n), cnt(n), nbr(n * (size_t)cap_);
  std::vector<uint8_t> mult(n * (size_t)cap_);
  if (n) {
    CK(cudaMemcpy(flags.data(), B.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(tags.data(), B.tag, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cnt.data(), B.ncnt, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nbr.data(), B.nbr, sizeof(uint32_t) * n * cap_, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(mult.data(), dbgMult_, n * (size_t)cap_, cudaMemcpyDeviceToHost));
  }
  std::vector<std::pair<uint32_t, size_t>> order;
  for (size_t k = 0; k < n; ++k)
    if (!(flags[k] & PF_DEAD)) order.emplace_back(tags[k], k);
  std::sort(order.begin(), order.end());
  std::vector<int64_t> id_of(n, -1);
  for (size_t i = 0; i < order.size(); ++i) id_of[order[i].second] = (int64_t)i;
  size_t c = 0;
  for (size_t k = 0; k < n; ++k) {
    if (id_of[k] < 0) continue;
    for (uint32_t m = 0; m < cnt[k]; ++m) {
      uint8_t v = mult[k * cap_ + m];
      if (!v) continue;
      if (pi && c < capacity) {
        pi[c] = id_of[k];
        pj[c] = id_of[nbr[k * cap_ + m]];
        visits[c] = v;
      }
      ++c;
    }
  }
  *nout = c;
  return RP_OK;
}

int Engine::debug_reference_grid(double h, int64_t* cell_of, int64_t* order, size_t* n_order, int32_t dims[3]) {
  TRY(ensure_gpu());
  if (!host_valid_) TRY(download());
  const size_t n = hp_.size();
  StepParams P = P_;
  P.href = h;
  P.inv_href = 1.0 / h;
  uint64_t ncells = 1;
  for (int k = 0; k < 3; ++k) {
    P.bmin[k] = bmin[k];
    double q = std::ceil((bmax[k] - bmin[k]) / h);
    if (!(q >= 0.0) || q > 1e7) {
      set_error("reference grid too large");
      return RP_E_INVALID_ARG;
    }
    P.rdims[k] = (int)q + 1;
    dims[k] = P.rdims[k];
    ncells *= (uint64_t)P.rdims[k];
  }
  if (ncells >= 0xFFFFFFF0ull) {
    set_error("reference grid too large");
    return RP_E_INVALID_ARG;
  }
  if (n == 0) {
    *n_order = 0;
    return RP_OK;
  }
  if (n > n_alloc_) {
    TRY(alloc_slots(n));
    dev_valid_ = false;  // slot buffers were re-allocated; the next step re-uploads
  }
  std::vector<D4> xr(n);
  for (size_t i = 0; i < n; ++i) xr[i] = D4{hp_[i].x[0], hp_[i].x[1], hp_[i].x[2], hp_[i].r};
  D4* xr_d = nullptr;
  TRY(dalloc(&xr_d, n));
  CK(cudaMemcpy(xr_d, xr.data(), sizeof(D4) * n, cudaMemcpyHostToDevice));
  int which = launch_reference_grid(P, xr_d, (int)n, (uint32_t)ncells, bits_for(ncells), kraw_, rb_.ka, rb_.va,
                                    rb_.kb, rb_.vb, rb_.hist, rb_.part, stream_);
  CK(cudaGetLastError());
  std::vector<uint32_t> raw(n), sk(n), sv(n);
  CK(cudaMemcpyAsync(raw.data(), kraw_, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, stream_));
  CK(cudaMemcpyAsync(sk.data(), which ? rb_.kb : rb_.ka, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, stream_));
  CK(cudaMemcpyAsync(sv.data(), which ? rb_.vb : rb_.va, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  cudaFree(xr_d);
  size_t m = 0;
  for (size_t i = 0; i < n; ++i) cell_of[i] = raw[i] >= ncells ? -1 : (int64_t)raw[i];
  for (size_t k = 0; k < n; ++k)
    if (sk[k] < ncells) order[m++] = (int64_t)sv[k];
  *n_order = m;
  // the device upload used the sort buffers: the next step rebuilds anyway
  return RP_OK;
}

// ------------------------------------------------------------- autotuner
// Chooses the force pass's launch shapes on the current state: the pass only
// reads the state and rewrites a, tau and its scratch buffers, so it can be
// timed repeatedly (CUDA events on the engine's stream, median of 5 after 2
// warm-up passes). Coordinate descent over the filter, pair and accumulate
// block sizes (64, 128, 256), the grid cap of their grid-stride loops, then the
// one-thread-per-particle path. The control block (counters, flags) is
// restored afterwards. Needs lists (a step already taken); the physical mode's
// spring history is rewritten by the pass, so that mode is not tuned.
int Engine::autotune(rp_tune_report* rep) {
  if (rep) std::memset(rep, 0, sizeof(*rep));
  TRY(ensure_gpu());
  if (!dev_valid_) {
    set_error("step at least once before autotuning (the force pass needs neighbour lists)");
    return RP_E_INVALID_ARG;
  }
  TRY(sync_ctrl());
  if (ctrl_h_->steps_done == 0 || ctrl_h_->rebuild || ctrl_h_->halt || n_ == 0) {
    set_error("step at least once before autotuning (the force pass needs neighbour lists)");
    return RP_E_INVALID_ARG;
  }
  if (mode == RP_MODE_PHYSICAL && tmodel != RP_TANGENTIAL_COULOMB) {
    set_error("the physical mode's spring history would change: not tuned");
    return RP_E_INVALID_ARG;
  }
  Ctrl saved;
  std::memcpy(&saved, ctrl_h_, sizeof(Ctrl));
  int tried = 0;
  auto time_pass = [&](float* out) -> int {
    for (int w = 0; w < 2; ++w) launch_force(P_, stream_);
    float t[5];
    for (int r = 0; r < 5; ++r) {
      CK(cudaEventRecord(ev0_, stream_));
      launch_force(P_, stream_);
      CK(cudaEventRecord(ev1_, stream_));
      CK(cudaEventSynchronize(ev1_));
      CK(cudaEventElapsedTime(&t[r], ev0_, ev1_));
    }
    CK(cudaGetLastError());
    std::sort(t, t + 5);
    *out = t[2];
    ++tried;
    return RP_OK;
  };
  const int nsm = P_.nsm;
  int cfg[5] = {0, 128, 128, 128, nsm * 64};  // path, filter, pair, accumulate, grid cap
  auto apply = [&](const int c[5]) {
    P_.force_path = c[0];
    P_.bs_filter = c[1];
    P_.bs_force = c[2];
    P_.bs_accum = c[3];
    P_.grid_cap = c[4];
  };
  apply(cfg);
  float best = 0.f;
  TRY(time_pass(&best));
  const float def_ms = best;
  const int blocks[3] = {64, 128, 256};
  const int caps[3] = {nsm * 4, nsm * 16, nsm * 64};
  for (int dim = 1; dim <= 4; ++dim) {
    for (int k = 0; k < 3; ++k) {
      int c[5];
      std::memcpy(c, cfg, sizeof(c));
      c[dim] = dim == 4 ? caps[k] : blocks[k];
      if (c[dim] == cfg[dim]) continue;
      apply(c);
      float t = 0.f;
      TRY(time_pass(&t));
      if (t < best) {
        best = t;
        std::memcpy(cfg, c, sizeof(c));
      }
    }
  }
  {
    int c[5];
    std::memcpy(c, cfg, sizeof(c));
    c[0] = 1;
    apply(c);
    float t = 0.f;
    TRY(time_pass(&t));
    if (t < best) {
      best = t;
      cfg[0] = 1;
    }
  }
  apply(cfg);
  force_path = cfg[0];
  bs_filter = cfg[1];
  bs_force = cfg[2];
  bs_accum = cfg[3];
  grid_cap = cfg[4];
  CK(cudaMemcpy(ctrl_, &saved, sizeof(Ctrl), cudaMemcpyHostToDevice));
  TRY(sync_ctrl());
  graph_dirty_ = true;
  if (rep) {
    rep->force_path = cfg[0];
    rep->bs_filter = cfg[1];
    rep->bs_force = cfg[2];
    rep->bs_accum = cfg[3];
    rep->grid_cap = cfg[4];
    rep->candidates = tried;
    rep->default_ms = def_ms;
    rep->best_ms = best;
  }
  return RP_OK;
}

// ------------------------------------------------------------ learned JKR
// Trains on the particle-pair domain of this simulation: R* between half the
// smallest and half the largest radius (or the given range), E* and gamma of
// the particle material scaled both ways, overlap/R* in [x_min, x_max].
int Engine::jkr_train(const rp_jkr_train_options* o, rp_jkr_train_report* rep) {
  rp_jkr_train_options d;
  std::memset(&d, 0, sizeof(d));
  if (o) d = *o;
  TRY(ensure_gpu());
  double rmin = 0.0, rmax = 0.0;
  if (!host_valid_) TRY(download());
  for (size_t i = 0; i < hp_.size(); ++i) {
    rmin = i == 0 ? hp_[i].r : std::min(rmin, hp_[i].r);
    rmax = std::max(rmax, hp_[i].r);
  }
  JkrTrainConfig cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.dom.rs_lo = d.rs_min > 0.0 ? d.rs_min : 0.5 * rmin;
  cfg.dom.rs_hi = d.rs_max > 0.0 ? d.rs_max : 0.5 * rmax;
  if (!(cfg.dom.rs_lo > 0.0) || !(cfg.dom.rs_hi >= cfg.dom.rs_lo)) {
    set_error("JKR training needs particles (or rs_min/rs_max) to fix the effective-radius range");
    return RP_E_INVALID_ARG;
  }
  if (cfg.dom.rs_hi <= cfg.dom.rs_lo) cfg.dom.rs_hi = cfg.dom.rs_lo * (1.0 + 1e-6);
  const double es = eff_youngs(pm.E, pm.nu, pm.E, pm.nu);
  const double gamma = (pm.gamma + pm.gamma) * 0.5;
  if (!(gamma > 0.0) || !(es > 0.0)) {
    set_error("JKR training needs a positive surface energy and Young's modulus");
    return RP_E_INVALID_ARG;
  }
  const double se = d.es_scale > 1.0 ? d.es_scale : 1.25, sg = d.gamma_scale > 1.0 ? d.gamma_scale : 1.25;
  cfg.dom.es_lo = es / se;
  cfg.dom.es_hi = es * se;
  cfg.dom.gamma_lo = gamma / sg;
  cfg.dom.gamma_hi = gamma * sg;
  cfg.dom.x_lo = (d.x_min == 0.0 && d.x_max == 0.0) ? -0.1 : d.x_min;
  cfg.dom.x_hi = (d.x_min == 0.0 && d.x_max == 0.0) ? 0.2 : d.x_max;
  if (!(cfg.dom.x_hi > cfg.dom.x_lo)) {
    set_error("x_max must exceed x_min");
    return RP_E_INVALID_ARG;
  }
  cfg.seed = d.seed ? d.seed : 1;
  cfg.n_samples = d.samples ? (size_t)d.samples : (size_t)1 << 20;
  cfg.epochs = d.epochs > 0 ? d.epochs : 24;
  cfg.batch = d.batch > 0 ? d.batch : 8192;
  cfg.lr0 = d.lr0 > 0.f ? d.lr0 : 3e-3f;
  cfg.lr1 = d.lr1 > 0.f ? d.lr1 : 2e-5f;
  cfg.qat_from_epoch = d.qat_from_epoch > 0 ? d.qat_from_epoch : (d.qat_from_epoch < 0 ? 0 : cfg.epochs / 2);
  cfg.n_val = 65536;
  if ((cfg.n_samples & (cfg.n_samples - 1)) != 0 || cfg.n_samples < 1024 || cfg.batch % 64 != 0 ||
      (size_t)cfg.batch > cfg.n_samples) {
    set_error("samples must be a power of two >= 1024 and batch a multiple of 64 not above it");
    return RP_E_INVALID_ARG;
  }
  JkrTrainResult* R = new (std::nothrow) JkrTrainResult;
  if (!R) return RP_E_NOMEM;
  const int rc = rp::jkr_train(cfg, R, stream_);
  if (rc != 0) {
    delete R;
    set_error("JKR network training failed (code %d)", rc);
    return RP_E_CUDA;
  }
  float dom[8];
  for (int k = 0; k < 4; ++k) {
    dom[k] = R->lo[k];
    dom[4 + k] = R->hi[k];
  }
  const int r2 = jkr_set_network(R->params, R->norm, dom);
  if (rep) {
    rep->final_loss = R->final_loss;
    rep->val_rms = R->val_rms;
    rep->val_max = R->val_max;
    rep->train_ms = R->train_ms;
    rep->samples = cfg.n_samples;
    rep->valid_samples = R->n_valid;
    rep->steps = R->steps;
  }
  delete R;
  return r2;
}

int Engine::jkr_set_network(const float* params, const float* norm, const float* domain) {
  for (int k = 0; k < MLP_NPARAM; ++k)
    if (!std::isfinite(params[k])) {
      set_error("network parameter %d is not finite", k);
      return RP_E_INVALID_ARG;
    }
  jkr_params_.assign(params, params + MLP_NPARAM);
  std::memcpy(jkr_norm_, norm, sizeof(jkr_norm_));
  std::memcpy(jkr_dom_, domain, sizeof(jkr_dom_));
  jkr_have_net_ = true;
  if (gpu_) dfree(mlp_d_);  // re-uploaded with the new weights
  dev_valid_ = false;
  return RP_OK;
}

int Engine::jkr_get_network(float* params, float* norm, float* domain) {
  if (!jkr_have_net_) {
    set_error("no JKR network installed");
    return RP_E_INVALID_ARG;
  }
  if (params) std::memcpy(params, jkr_params_.data(), sizeof(float) * MLP_NPARAM);
  if (norm) std::memcpy(norm, jkr_norm_, sizeof(jkr_norm_));
  if (domain) std::memcpy(domain, jkr_dom_, sizeof(jkr_dom_));
  return RP_OK;
}

int Engine::jkr_counters(uint64_t out[6]) {
  for (int k = 0; k < 6; ++k) out[k] = 0;
  if (!gpu_ || !dev_valid_) return RP_OK;
  CK(cudaSetDevice(device_));
  TRY(sync_ctrl());
  for (int k = 0; k < 6; ++k) out[k] = ctrl_h_->jkr_count[k];
  return RP_OK;
}

}  // namespace rp
