// Host engine behind the C ABI: owns the particle store, the device buffers
// and the step sequencing. Mirrors the reference's `Simulation` struct
// (src/simulation.rs:16-51) with GPU-resident state.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rp.h"
#include "rp_device.cuh"
#include "rp_launch.h"
#include "rp_mlp.cuh"

namespace rp {

struct HostParticle {
  double x[3], v[3], a[3], w[3], tau[3], xres[3], vres[3], wres[3];
  double r, m;
  uint8_t fixed;
  uint32_t tag;
  uint32_t group;  // independent bed (0 unless set)
};

struct Totals {
  uint64_t steps = 0, removed = 0, rebuilds = 0, overlap_steps = 0, status = 0, max_count = 0;
};

class Engine {
 public:
  Engine(double dt, const double mn[3], const double mx[3], size_t capacity);
  ~Engine();

  // configuration (src/simulation.rs:62-91 defaults)
  double dt;
  double bmin[3], bmax[3];
  int periodic[3] = {0, 0, 0};
  Material pm{1e7, 0.3, 2500.0, 0.5, 0.5, 0.0};
  Material wm{1e9, 0.3, 7800.0, 0.5, 0.5, 0.0};
  int nmodel = RP_NORMAL_HERTZ, tmodel = RP_TANGENTIAL_MINDLIN;
  int mode = RP_MODE_PARITY, prec = RP_PREC_FP64;
  double gravity[3] = {0.0, -9.81, 0.0};
  double href = 1.0;
  double skin_user = -1.0;
  int debug = 0;
  int profiling = 0;
  int force_path = 0;  // 0 contact-parallel, 1 one thread per particle

  int add_particle(const double x[3], double r, double m, int fixed);
  // n particles at once; appended to the device slots without a host round
  // trip while the device holds the state (see append_on_device)
  int add_particles(size_t n, const double* xyz, const double* r, const double* m, const uint8_t* fixed);
  int add_triangles(size_t n, const float* v, const float* nrm, uint32_t group = GROUP_ALL,
                    const WallMotion* motion = nullptr);
  // groups: independent beds stepped together
  int set_particle_groups(size_t n, const uint32_t* groups);
  int get_particle_groups(size_t n, uint32_t* groups);
  int set_group_material(uint32_t group, const Material& m);
  Law make_law(const Material& m) const;
  // launch shapes of the force pass (0 = default) and their autotuner
  int bs_filter = 0, bs_force = 0, bs_accum = 0, grid_cap = 0;
  int autotune(rp_tune_report* rep);
  int enable_gpu(int device);
  int step(uint64_t n);
  size_t count();
  int get_vec(size_t id, int which, double out[3]);
  int set_vec(size_t id, int which, const double in[3]);
  int read_state(rp_state* st);
  int write_state(const rp_state* st);
  int stats(rp_stats* st);
  int bed_statistics(double out[3]);
  int debug_forces(double* F, double* T);
  int debug_pairs(int64_t* pi, int64_t* pj, int32_t* visits, size_t capacity, size_t* n);
  int debug_reference_grid(double h, int64_t* cell_of, int64_t* order, size_t* n_order, int32_t dims[3]);
  int debug_triangle_grid(int32_t dims[3], double lo_cell[4], uint32_t* start, size_t start_cap, uint32_t* items,
                          size_t items_cap, size_t* n_start, size_t* n_items);
  bool tgrid_built_ = false;
  int write_vtk(const char* path);
  // learned JKR (RP_JKR_*)
  int jkr_solver = RP_JKR_NEWTON;
  int jkr_train(const rp_jkr_train_options* o, rp_jkr_train_report* rep);
  int jkr_set_network(const float* params, const float* norm, const float* domain);
  int jkr_get_network(float* params, float* norm, float* domain);
  bool jkr_has_network() const { return jkr_have_net_; }
  int jkr_counters(uint64_t out[6]);
  void config_changed() { dev_valid_ = false; }  // forces a fresh upload before the next step
  void set_capacity(int c) {
    if (!host_valid_) download();
    free_lists();
    cap_ = c;
    dev_valid_ = false;
  }

 private:
  std::vector<HostParticle> hp_;  // id order when host_valid_
  std::vector<uint32_t> up_tags_;  // insertion tags of the uploaded particles; a slot's device tag indexes it
  bool host_valid_ = true, dev_valid_ = false;
  uint32_t next_tag_ = 0;
  std::vector<float> tri_v_, tri_n_;
  std::vector<uint32_t> tri_group_;  // per triangle (GROUP_ALL unless given)
  std::vector<uint32_t> tri_motion_;  // per triangle (NO_MOTION unless given)
  std::vector<WallMotion> motions_;
  WallMotion* motions_d_ = nullptr;
  std::vector<Material> gmat_;       // per group (index 0 unused: the particle material)
  std::vector<uint8_t> gmat_set_;
  Law* glaw_d_ = nullptr;
  double ms_total_ = 0.0;
  uint64_t launches_ = 0;
  uint64_t force_launches_ = 0;
  double force_ms_ = 0.0;
  std::vector<cudaEvent_t> fev_;  // force-kernel event pairs (profiling)
  // device step loop (CUDA graph with WHILE and IF conditional nodes)
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  cudaStream_t cap_stream_ = nullptr, cap_stream2_ = nullptr;
  bool graph_dirty_ = true;
  int chain_kernels_ = 0;

 public:
  bool use_graph_ = true;

 private:

  // device
  bool gpu_ = false;
  int device_ = -1;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  size_t n_alloc_ = 0;  // slots allocated
  int cap_ = 0;         // neighbour list capacity per slot
  int n_ = 0;           // slots in use
  Bank bank_[2] = {};
  Ctrl* ctrl_ = nullptr;
  Ctrl* ctrl_h_ = nullptr;  // pinned mirror
  Ctrl last_ = {};
  Totals tot_;
  RebuildBufs rb_ = {};
  uint32_t* kraw_ = nullptr;
  size_t fcells_alloc_ = 0;
  double* dbgF_ = nullptr;
  double* dbgT_ = nullptr;
  uint8_t* dbgMult_ = nullptr;
  // contact-parallel force buffers
  CRec* crec_ = nullptr;
  uint32_t *ccnt_ = nullptr, *coff_ = nullptr, *clist_ = nullptr;
  uint32_t* aorder_ = nullptr;  // k_accumulate visiting order (set at every list rebuild)
  uint2* warena_ = nullptr;     // wall candidates of the force pass
  double* wres_ = nullptr;      // their results
  uint8_t* wok_ = nullptr;      // their contact flags
  uint32_t *woff_ = nullptr, *wcnt_ = nullptr;
  size_t wcap_ = 0;
  uint32_t *ctot_ = nullptr;
  double* cres_ = nullptr;
  void refresh_list_ptrs();
  double* ke_ = nullptr;
  // learned JKR: installed network and its per-step queue
  bool jkr_have_net_ = false;
  std::vector<float> jkr_params_;
  float jkr_norm_[10] = {};
  float jkr_dom_[8] = {};
  MlpInfer* mlp_d_ = nullptr;
  uint2* jq_ = nullptr;
  float* jguess_ = nullptr;
  size_t jq_alloc_ = 0;
  uint32_t* jfb_ = nullptr;  // pairs deferred to the reference-Newton pass
  size_t jfb_alloc_ = 0;
  int ensure_jkr_buffers();
  int step_kernels_ = 4;  // kernels of one device-loop step outside the rebuild chain
  TriRec* tri_d_ = nullptr;
  uint32_t *tstart_d_ = nullptr, *titems_d_ = nullptr;
  StepParams P_ = {};
  std::vector<unsigned char> stage_;  // host staging

  int ensure_gpu();
  int upload();
  int download();
  // device-side removal and insertion (src/simulation.rs:199-219, 93-96)
  int compact_removed();
  int append_on_device(size_t n, const double* xyz, const double* r, const double* m, const uint8_t* fixed,
                       bool& done);
  int n_upload_ = 0;          // upload positions (device tags index them); > n_ after compactions
  double rmax_dev_ = 0.0;     // largest radius of the uploaded set (sizes the grids)
  uint64_t uploads_ = 0, downloads_ = 0, compactions_ = 0, device_inserts_ = 0;
  // bulk state in id order straight between the caller's arrays and the slots
  // (valid device state, no dead slot); `done` is false when it does not apply
  int fast_read_state(rp_state* st, bool& done);
  int fast_write_state(const rp_state* st, bool& done);
  int ensure_io(size_t n);
  double* io_buf_ = nullptr;   // staging: 8 x 3n vectors, radius, mass, fixed
  bool io_direct_ = false;     // kernels reach the caller's pageable arrays (host page tables)
  size_t io_n_ = 0;
  uint32_t* slot_of_ = nullptr;
  uint32_t *id_live_ = nullptr, *id_pos_ = nullptr, *slot_of_id_ = nullptr, *id_part_ = nullptr;
  unsigned* io_flag_ = nullptr;
  int alloc_slots(size_t n);
  int alloc_lists(int cap, bool keep_current);
  int build_params();
  int build_triangle_grid(double rmax);
  void free_device();
  void free_lists();
  int launch_steps(uint64_t n);
  int launch_steps_graph(uint64_t n);
  int build_graph();
  void destroy_graph();
  int recover_halt();
  int alloc_walls(size_t cap);
  int sync_ctrl();
  int finish_step_accounting();
};

}  // namespace rp
