/*
 * rp.h — C ABI of the GB300 DEM step (librp.so).
 *
 * The reference exposes its engine only through a pyo3 extension module,
 * `rusty_particles` (src/lib.rs:24-35), whose class `Simulation`
 * (src/lib.rs:41-277) owns a Rust `simulation::Simulation`
 * (src/simulation.rs:16-51). This header is the flat C boundary a binding
 * (ctypes, cgo, a Rust `extern "C"` block, JNI) calls in its place. Every
 * entry point below names the reference interface it replaces.
 *
 * Conventions
 *   - Plain pointers and sizes only; no CUDA or torch types cross the ABI.
 *   - Return codes: RP_OK (0) or a negative RP_E_* code. rp_last_error()
 *     returns the message of the last failure on the calling thread.
 *   - A handle is owned by one host thread at a time (like the reference's
 *     `&mut self` methods); distinct handles are independent.
 *   - Particle ids are indices in insertion order after removals, exactly as
 *     the reference re-indexes (src/simulation.rs:216-219).
 *   - All stepping runs on the GPU. There is no CPU fallback: without a
 *     usable CUDA device, rp_enable_gpu / rp_step / rp_run fail with RP_E_CUDA.
 */
#ifndef RP_H
#define RP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RP_OK 0
#define RP_E_INVALID_ARG (-1) /* maps to Python ValueError */
#define RP_E_INDEX (-2)       /* maps to Python IndexError */
#define RP_E_IO (-3)          /* maps to Python IOError */
#define RP_E_CUDA (-4)        /* maps to Python RuntimeError */
#define RP_E_DEVICE_FLAG (-5) /* device reported a condition it could not recover from */
#define RP_E_TIMEOUT (-6)     /* a bounded device-side wait ran out */
#define RP_E_NOMEM (-7)       /* host or device allocation failed */

/* Normal force models, in the reference enum order (src/physics.rs:6-17). */
#define RP_NORMAL_LINEAR 0
#define RP_NORMAL_HERTZ 1
#define RP_NORMAL_HYSTERETIC 2
#define RP_NORMAL_JKR 3
#define RP_NORMAL_SJKR 4
/* Tangential force models, in the reference enum order (src/physics.rs:21-28). */
#define RP_TANGENTIAL_COULOMB 0
#define RP_TANGENTIAL_LINEAR_SPRING 1
#define RP_TANGENTIAL_MINDLIN 2

/* Arithmetic of the pair forces. State, accumulation and the integrator are
 * FP64 in both modes. */
#define RP_PREC_FP64 0  /* all pair math in FP64 */
#define RP_PREC_MIXED 1 /* pair math in FP32 on FP64-differenced inputs */

/* Interaction rules. */
#define RP_MODE_PARITY 0   /* the reference's rules, including its defects */
#define RP_MODE_PHYSICAL 1 /* minimum-image pairs once each, Mindlin G*, history per pair */

typedef struct rp_sim rp_sim;

/* Host-side state view used by rp_read_state / rp_write_state. Arrays are in
 * particle-id order; vectors hold 3 doubles per particle. Any pointer may be
 * NULL (that field is skipped). n_particles is the length of the caller's
 * arrays and must equal rp_particle_count(); both calls reject any other value
 * with RP_E_INVALID_ARG before touching an array. */
typedef struct rp_state {
  size_t n_particles;
  double* position;         /* 3N */
  double* velocity;         /* 3N */
  double* angular_velocity; /* 3N */
  double* acceleration;     /* 3N */
  double* torque;           /* 3N */
  double* position_residual;
  double* velocity_residual;
  double* angular_velocity_residual;
  double* radius;  /* N */
  double* mass;    /* N */
  uint8_t* fixed;  /* N */
} rp_state;

typedef struct rp_stats {
  uint64_t steps;              /* steps completed on this handle */
  uint64_t particles;          /* current particle count */
  uint64_t removed;            /* particles removed by the out-of-bounds rule */
  uint64_t neighbor_rebuilds;  /* Verlet-list rebuilds */
  uint64_t overlap_warn_steps; /* steps with an overlap > 20 % of a radius */
  uint64_t status_bits;        /* RP_STATUS_* seen since creation */
  uint64_t neighbor_capacity;  /* list slots per particle */
  uint64_t max_neighbors;      /* longest list at the last rebuild */
  double kinetic_energy;       /* FP64, translational + rotational, at the last rp_get_stats */
  double device_ms;            /* device time of the stepping calls so far */
  uint64_t kernel_launches;    /* kernels launched by stepping calls so far */
  uint64_t force_launches;     /* force-kernel launches timed (profiling on) */
  double force_ms;             /* their summed device time (CUDA events on the launching stream) */
  uint64_t state_io_direct;    /* 1: rp_read_state / rp_write_state move bulk state by kernels on
                                  the caller's pageable arrays (the device reaches host memory through
                                  the host page tables; opt-in, RP_DIRECT_STATE_IO=1); 0: staged
                                  device copies (default) */
  uint64_t state_uploads;      /* full host->device uploads of the particle state (first step, host edits) */
  uint64_t state_downloads;    /* full device->host downloads of the particle state (per-particle getters) */
  uint64_t compactions;        /* removals compacted on the device (no host round trip) */
  uint64_t device_inserts;     /* particles appended to the device slots without a host round trip */
} rp_stats;

#define RP_STATUS_OVERLAP 1u    /* overlap > 20 % of the smaller radius (src/simulation.rs:361-370) */
#define RP_STATUS_NAN_FORCE 2u  /* a non-finite particle force */
#define RP_STATUS_NLIST_GROW 4u /* a neighbour list outgrew its capacity (recovered) */
#define RP_STATUS_WALL_GROW 8u  /* the wall contact candidates outgrew their buffer (recovered) */

/* --- lifecycle: Simulation.create (src/lib.rs:57, src/simulation.rs:62-91) */
rp_sim* rp_create(double dt, const double min_xyz[3], const double max_xyz[3], size_t particle_capacity);
void rp_destroy(rp_sim* sim);

/* --- Simulation.add_particle (src/lib.rs:76-80, src/simulation.rs:93-96) */
int rp_add_particle(rp_sim* sim, double x, double y, double z, double radius, double mass, int fixed);
/* Bulk form of rp_add_particle: n particles, xyz holds 3n doubles; fixed may be NULL. */
int rp_add_particles(rp_sim* sim, size_t n, const double* xyz, const double* radius, const double* mass,
                     const uint8_t* fixed);

/* --- Simulation.add_mesh (src/lib.rs:87-91, src/mesh.rs:125-143): binary or ASCII STL */
int rp_add_mesh_stl(rp_sim* sim, const char* path);
/* Triangles given directly: 9 floats per triangle (v0,v1,v2) and 3 per normal
 * (NULL computes (v1-v0)x(v2-v0) normalised). */
int rp_add_mesh_triangles(rp_sim* sim, size_t n_triangles, const float* vertices, const float* normals);

/* --- Simulation.set_particle_material / set_wall_material (src/lib.rs:98-129) */
int rp_set_particle_material(rp_sim* sim, double youngs_modulus, double poissons_ratio, double density,
                             double friction_coefficient, double restitution_coefficient, double surface_energy);
int rp_set_wall_material(rp_sim* sim, double youngs_modulus, double poissons_ratio, double density,
                         double friction_coefficient, double restitution_coefficient, double surface_energy);

/* --- Simulation.set_contact_models (src/lib.rs:160-180) */
int rp_set_contact_models(rp_sim* sim, int normal_model, int tangential_model);
/* The reference's case-insensitive name table (src/lib.rs:163-175); returns
 * RP_E_INVALID_ARG for an unknown name. */
int rp_parse_contact_models(const char* normal, const char* tangential, int* normal_model, int* tangential_model);

/* --- Simulation.set_periodic_boundary (src/lib.rs:138) */
int rp_set_periodic(rp_sim* sim, int x, int y, int z);

/* --- Simulation.enable_gpu (src/lib.rs:146-148, src/simulation.rs:129-146):
 * selects CUDA device `device` (-1 = current) and uploads the particles. */
int rp_enable_gpu(rp_sim* sim, int device);

/* --- Simulation.step / run (src/lib.rs:94, 182-195, src/simulation.rs:156-171) */
int rp_step(rp_sim* sim, uint64_t n_steps);
/* steps = ceil(duration / dt) evaluated in f32, as src/lib.rs:356 does. */
int rp_run(rp_sim* sim, double duration);

/* --- getters and setters (src/lib.rs:210-276); id out of range -> RP_E_INDEX */
size_t rp_particle_count(rp_sim* sim);
int rp_get_particle_position(rp_sim* sim, size_t id, double out_xyz[3]);
int rp_get_particle_velocity(rp_sim* sim, size_t id, double out_xyz[3]);
int rp_get_particle_angular_velocity(rp_sim* sim, size_t id, double out_xyz[3]);
int rp_set_particle_velocity(rp_sim* sim, size_t id, double vx, double vy, double vz);
int rp_set_particle_angular_velocity(rp_sim* sim, size_t id, double wx, double wy, double wz);

/* --- Simulation.write_vtk (src/lib.rs:202-207, src/vtk.rs:5-44) */
int rp_write_vtk(rp_sim* sim, const char* path);

/* --- bulk state transfer (no reference counterpart; replaces the wgpu
 * upload/readback of src/gpu.rs:92-98 and src/gpu.rs:168-213) */
int rp_read_state(rp_sim* sim, rp_state* out);
int rp_write_state(rp_sim* sim, const rp_state* in);

/* --- options with the reference's hard-coded values as defaults */
int rp_set_precision(rp_sim* sim, int precision);        /* RP_PREC_*; default FP64 */
int rp_set_interaction_mode(rp_sim* sim, int mode);      /* RP_MODE_*; default PARITY */
int rp_set_gravity(rp_sim* sim, double gx, double gy, double gz); /* default (0,-9.81,0), src/simulation.rs:267 */
int rp_set_reference_cell_size(rp_sim* sim, double h);   /* default 1.0, src/simulation.rs:66 */
int rp_set_skin(rp_sim* sim, double skin);               /* Verlet skin; <= 0 selects the default */
int rp_set_neighbor_capacity(rp_sim* sim, int capacity); /* initial list slots per particle (grows on demand) */
/* 1 (default): a stepping call is one CUDA-graph launch whose device-side loop
 * runs all steps and rebuilds lists only when needed; 0: the host issues the
 * kernels step by step in chunks. */
int rp_set_device_loop(rp_sim* sim, int enable);
/* Force evaluation: 0 (default) contact-parallel (filter per particle, one
 * thread per contact pair, per-particle sum in list order); 1 one thread per
 * particle over its whole list. Same results within rounding. */
int rp_set_force_path(rp_sim* sim, int path);
int rp_set_threads(int n);                               /* set_num_threads (src/lib.rs:15-22) */

/* --- metrics and errors */
int rp_get_stats(rp_sim* sim, rp_stats* out);
/* Statistics of the bed in its current state, in FP64 on the device (no
 * reference counterpart; the reference's scripts compute them in Python):
 * out[0] kinetic energy, translational plus rotational with I = 2/5 m r^2;
 * out[1] coordination number, 2 x (pairs with |d| < r_i + r_j, minimum image
 * on periodic axes) / particles; out[2] solid fraction of the simulation box,
 * the spheres' summed volume over the box volume. Needs one completed step
 * (the pair count runs over the neighbour lists). */
int rp_bed_statistics(rp_sim* sim, double out[3]);
/* Time every force-kernel launch with CUDA events (adds two event records per step). */
int rp_set_profiling(rp_sim* sim, int enable);
const char* rp_last_error(void);
const char* rp_version(void);

/* FP64 throughput of the current device, measured with CUDA events (thread
 * instructions per second of FP64 fused multiply-add and of FP64 addition,
 * eight independent chains per thread, best of three launches): the ceiling of
 * the FP64-bound kernels of the step. No reference counterpart. */
int rp_measure_fp64_peak(double* fma_per_s, double* add_per_s);

/* --- diagnostics for parity checks (no reference counterpart) */
/* Record per-particle force/torque and contact multiplicities during steps. */
int rp_set_debug(rp_sim* sim, int enable);
/* Per-particle (f_total, torque_total) of the last step, before division by
 * mass (src/simulation.rs:317-526), in id order; 3N doubles each. */
int rp_debug_last_forces(rp_sim* sim, double* force, double* torque);
/* Contact pairs of the last step seen from particle i: (i, j, visits) with
 * visits the number of times the reference's loop would visit j
 * (src/simulation.rs:322-357). Returns the pair count in *n; pass NULL arrays
 * to query the count. */
int rp_debug_contact_pairs(rp_sim* sim, int64_t* pi, int64_t* pj, int32_t* visits, size_t capacity, size_t* n);
/* Runs the device cell-hash + radix-sort chain with the reference grid
 * (src/grid.rs:12-46: cell size h, origin min, dims = ceil(size/h)+1) on the
 * current positions. cell_of[i] = linear cell of particle i or -1 if outside
 * the grid; order[] = particle ids grouped by cell, stable in id order
 * (the flattened `cells` vectors); *n_order = number of inserted particles. */
int rp_debug_reference_grid(rp_sim* sim, double h, int64_t* cell_of, int64_t* order, size_t* n_order,
                            int32_t dims[3]);
/* The triangle grid of the wall contacts as built on the device (replaces the
 * every-triangle loop of src/simulation.rs:464-523 with the triangles of the
 * centre's cell, in mesh order): dims, lo_cell = {origin x, y, z, cell size},
 * start[c] (ncells + 1 entries; *n_start receives ncells + 1) and the triangle
 * ids of cell c at items[start[c] .. start[c+1]) (*n_items receives their
 * count). Arrays shorter than needed are left untouched (query with NULL).
 * Uploads the state first when the device does not hold it. */
int rp_debug_triangle_grid(rp_sim* sim, int32_t dims[3], double lo_cell[4], uint32_t* start, size_t start_cap,
                           uint32_t* items, size_t items_cap, size_t* n_start, size_t* n_items);

/* --- groups: independent beds stepped together (no counterpart in the
 * reference, which simulates one bed per Simulation). A group is what one
 * reference Simulation would hold: its particles interact only with each other
 * and with the group's triangles (or those added for all groups), under the
 * group's particle material; dt, models, gravity, bounds and the wall
 * material are shared. Group 0 uses rp_set_particle_material. With every
 * particle in group 0 (the default) nothing changes. */
#define RP_GROUP_ALL 0xFFFFFFFFu
/* groups[i] for particle id i (n = rp_particle_count), each < 2^24. */
int rp_set_particle_groups(rp_sim* sim, size_t n, const uint32_t* groups);
int rp_get_particle_groups(rp_sim* sim, size_t n, uint32_t* groups);
/* The particle material of one group (as rp_set_particle_material). */
int rp_set_group_material(rp_sim* sim, uint32_t group, double youngs_modulus, double poissons_ratio, double density,
                          double friction_coefficient, double restitution_coefficient, double surface_energy);
/* rp_add_mesh_triangles for the particles of one group (RP_GROUP_ALL: every group). */
int rp_add_mesh_triangles_group(rp_sim* sim, size_t n_triangles, const float* vertices, const float* normals,
                                uint32_t group);

/* --- moving walls (no counterpart in the reference, whose walls are static):
 * triangles whose surface moves with velocity + omega x (p - center) while the
 * geometry stays (a drum turning about its own axis, a belt). The wall enters
 * each contact's relative velocity at the contact point. */
int rp_add_mesh_triangles_moving(rp_sim* sim, size_t n_triangles, const float* vertices, const float* normals,
                                 uint32_t group, const double center[3], const double omega[3],
                                 const double velocity[3]);

/* --- launch shapes of the force pass (no counterpart in the reference) */
typedef struct rp_tune_report {
  int32_t force_path; /* 0 contact-parallel, 1 one thread per particle */
  int32_t bs_filter, bs_force, bs_accum; /* threads per block */
  int32_t grid_cap;   /* largest grid of the grid-stride loops */
  int32_t candidates; /* configurations timed */
  double default_ms, best_ms; /* median force-pass time, default and chosen shape */
} rp_tune_report;
/* Times the force pass on the current state for candidate shapes (block
 * sizes 64/128/256 per kernel, grid caps, the per-particle path) and keeps
 * the fastest. The state is not changed. Needs one completed step; not
 * available in physical mode with a spring history. report may be NULL. */
int rp_autotune(rp_sim* sim, rp_tune_report* report);
/* Sets the shapes directly (0 = default: 128 threads, 64 blocks per multiprocessor). */
int rp_set_launch_shape(rp_sim* sim, int bs_filter, int bs_force, int bs_accum, int grid_cap);

/* --- learned JKR contact radius (no counterpart in the reference; replaces
 * the per-contact Newton iteration of src/physics.rs:164-191 for particle
 * pairs of the JKR model)
 *
 * Solvers (rp_set_jkr_solver):
 *   RP_JKR_NEWTON  the reference's Newton iteration (default)
 *   RP_JKR_LEARNED exact certificates decide pairs where the reference returns
 *                  zero or provably converges; the latter take a/R* from a
 *                  4-64-64-64-1 network (BF16 weights, FP32 accumulation, on
 *                  the tensor cores), two FP32 Newton steps, an FP64 residual
 *                  check (relative residual > 1e-6 -> the reference's Newton)
 *                  and one FP64 correction. Needs a network (rp_jkr_train or
 *                  rp_jkr_set_network).
 *   RP_JKR_CERTIFIED the same certificates and checks without the network
 *                  (FP32 Newton from the reference's start): the method
 *                  without its learned part. */
#define RP_JKR_NEWTON 0
#define RP_JKR_LEARNED 1
#define RP_JKR_CERTIFIED 2
#define RP_MLP_PARAMS 8705 /* FP32 parameters: W1[64][4] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4 */

typedef struct rp_jkr_train_options {
  double rs_min, rs_max;  /* effective radius range; 0 = r_min/2 .. r_max/2 of the particles */
  double es_scale;        /* E* sampled log-uniform from E* over s to E* times s; 0 = 1.25 */
  double gamma_scale;     /* surface energy likewise; 0 = 1.25 */
  double x_min, x_max;    /* overlap / R* range; both 0 = [-0.1, 0.2] */
  uint64_t seed;          /* 0 = 1 */
  uint64_t samples;       /* power of two; 0 = 1,048,576 */
  int32_t epochs;         /* 0 = 24 */
  int32_t batch;          /* multiple of 64; 0 = 8192 */
  float lr0, lr1;         /* cosine schedule; 0 = 3e-3 .. 2e-5 */
  int32_t qat_from_epoch; /* quantisation-aware from this epoch; 0 = epochs / 2, < 0 = from the start */
} rp_jkr_train_options;

typedef struct rp_jkr_train_report {
  double final_loss;    /* last mini-batch loss (normalised target) */
  double val_rms;       /* held-out error of the BF16 network in t = ln(a/R*) - ln sqrt(max(x,0)+c^(2/3)) */
  double val_max;
  double train_ms;      /* wall time of sample generation + training */
  uint64_t samples, valid_samples, steps;
} rp_jkr_train_report;

/* Generates samples with the reference's Newton solver on the GPU, trains the
 * network there with the project's forward/backward/Adam kernels, and installs
 * it in the simulation. options/report may be NULL. Material and radii must
 * be set before the call. */
int rp_jkr_train(rp_sim* sim, const rp_jkr_train_options* options, rp_jkr_train_report* report);
int rp_set_jkr_solver(rp_sim* sim, int solver);
/* The installed network: params[RP_MLP_PARAMS], norm[10] (feature mean[4],
 * 1/std[4], target mean, std), domain[8] (raw-feature min[4], max[4]). */
int rp_jkr_get_network(rp_sim* sim, float* params, float* norm, float* domain);
int rp_jkr_set_network(rp_sim* sim, const float* params, const float* norm, const float* domain);
/* Pair evaluations since the last upload: [0] accepted by the certified solver,
 * [1] certified zero, [2] reference-Newton fallbacks, [3] network rows used,
 * [4] FP32 Newton steps, [5] pairs decided by the closed-form walk. */
int rp_jkr_counters(rp_sim* sim, uint64_t out[6]);

/* Building blocks of the learned solver, on the current CUDA device (host
 * buffers in and out). Features and targets are normalised. */
/* Loss sum_s w_s (y_s - t_s)^2 / n and its gradient for n samples (n a power
 * of two, >= 64); qat = 1 evaluates the forward pass as inference does (BF16
 * weights and layer inputs, tanh.approx) with straight-through gradients. */
int rp_mlp_loss_grad(const float* params, const float* features, const float* targets, const float* weights, size_t n,
                     int qat, float* grad, double* loss);
/* Tensor-core inference (BF16 weights rounded to nearest even) on n rows. */
int rp_mlp_infer(const float* params, const float* features, size_t n, float* out);
/* Training samples: domain = {rs_lo, rs_hi, E*_lo, E*_hi, gamma_lo, gamma_hi,
 * x_lo, x_hi}; writes raw features (4n), target t (n), weight (n, 1 where the
 * network applies), the reference Newton's a (n, may be NULL) and its loop
 * count (n, may be NULL; negative where the pair is not network-eligible),
 * and the FP64 inputs (overlap, R*, E*, gamma) of each sample (4n, may be
 * NULL). */
int rp_jkr_samples(const double domain[8], uint64_t seed, size_t n, float* features, float* targets, float* weights,
                   double* a_ref, int32_t* iters, double* inputs);

/* --- allocation-free cell sort (no counterpart in the reference)
 * For callers that cannot call cudaMalloc: code issuing work inside a CUDA
 * stream capture, engines whose pool allocator owns all device memory, and
 * real-time loops that cannot afford cudaMalloc's device synchronisation.
 * Same result as rp_debug_reference_grid's hash + stable radix sort, on
 * caller-owned DEVICE buffers: positions (3n doubles), origin/cell_size/dims
 * of the grid (the reference's formula, src/grid.rs:30-40); writes
 * cell_of[i] (linear cell, or 0xFFFFFFFF outside the grid) and order[] (all n
 * particle indices sorted by cell, stable in index order, outside ones last),
 * on `stream` (a cudaStream_t; NULL = legacy default stream), asynchronously.
 * Its temporaries live in one static device array sized for at most 262,144
 * particles (larger n -> RP_E_INVALID_ARG); it calls no cudaMalloc/cudaFree.
 * The array is shared by every call: calls that overlap on the GPU race and
 * must be serialised by the caller. The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture. That address is cached for the life of the process and
 * belongs to the device's current context: after cudaDeviceReset (or any other
 * teardown of that context) the cache is stale, so do not call this entry
 * point again in a process that has reset the device. */
int rp_cell_sort_noalloc(const double* positions, size_t n, const double origin[3], double cell_size,
                         const int32_t dims[3], uint32_t* cell_of, uint32_t* order, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RP_H */
