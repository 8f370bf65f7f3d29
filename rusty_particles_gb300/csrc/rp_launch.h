// Host-side launch interface of the device kernels (one header for the
// translation units that launch and the engine that sequences them).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "rp_device.cuh"

namespace rp {

// Multiprocessors of the current CUDA device (cudaDevAttrMultiProcessorCount,
// looked up once per device; 152 on GB300).
int sm_count();

inline int grid_for(uint64_t n, int block) {
  uint64_t g = (n + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 64ull;  // grid-stride loops cover the rest
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

struct RebuildBufs {
  uint32_t *ka, *va, *kb, *vb;  // sort ping-pong
  uint32_t* hist;               // radix digit histograms
  uint32_t* part;               // scan partials
  uint32_t *cstart, *cend;      // fine-cell bounds
  int key_bits;
  int carry_history;
};

// k_broadphase.cu
void launch_exclusive_scan(const Ctrl* gate, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* part,
                           uint32_t* total, cudaStream_t s);
uint32_t scan_parts_needed(uint32_t n);
uint32_t radix_hist_needed(uint32_t n);
int launch_radix_sort(const Ctrl* gate, uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, uint32_t n, int bits,
                      uint32_t* hist, uint32_t* part, cudaStream_t s);
int launch_rebuild(const StepParams& P, const RebuildBufs& R, cudaStream_t s);  // returns kernels launched
int launch_reference_grid(const StepParams& P, const D4* xr, int n, uint32_t ncells, int key_bits, uint32_t* kraw,
                          uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, uint32_t* hist, uint32_t* part,
                          cudaStream_t s);

// k_trigrid.cu: the triangle grid of the wall contacts. The host passes each
// triangle's cell box (a0 a1 a2 b0 b1 b2, ints) and the exclusive scan of the
// box sizes (coff, T+1 entries, total = coff[T]); the device writes the
// triangle records, sorts the kept (cell, triangle) candidates and writes
// tstart (ncells+1 entries); *items points at the triangle ids in cell order
// (ka/va/kb/vb/hist/part are sort buffers for `total` keys, counts ncells+1).
struct TriGridShape {
  double lo[3];
  double cell;
  int dims[3];
  uint32_t ncells;
  double reach2;  // a cell whose centre is farther than sqrt(reach2) from a triangle does not list it
};
int launch_triangle_grid(const float* v, const float* nrm, const uint32_t* grp, const uint32_t* mot, int T,
                         const int* box, const uint32_t* coff, uint32_t total, const TriGridShape& S,
                         TriRec* recs, uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, uint32_t* hist,
                         uint32_t* part, uint32_t* counts, uint32_t* tstart, cudaStream_t s, const uint32_t** items);

// k_step.cu
int launch_first_half(const StepParams& P, cudaStream_t s);  // each returns kernels launched
int launch_second_half(const StepParams& P, cudaStream_t s);
int launch_rebuild_condition(const StepParams& P, cudaGraphConditionalHandle h, cudaStream_t s);
int launch_end_step_loop(const StepParams& P, cudaGraphConditionalHandle loop, cudaStream_t s);
int launch_force(const StepParams& P, cudaStream_t s);
int launch_accum_order(const StepParams& P, cudaStream_t s);  // inside the rebuild chain, before the bank flip
int launch_end_step(const StepParams& P, cudaStream_t s);
// Kinetic energy (translational + rotational) of the live slots, FP64.
void launch_kinetic_energy(const StepParams& P, double* out, cudaStream_t s);
// Bed statistics: out[0] kinetic energy, out[1] summed sphere volumes (both
// FP64), *pairs overlapping pairs counted from both ends (needs current lists).
void launch_bed_stats(const StepParams& P, double* out, unsigned long long* pairs, cudaStream_t s);

// Bulk state transfer in id order (ids of the live particles): the eight vector arrays of
// rp_state in the order position, velocity, angular velocity, acceleration,
// torque and the three residuals (3 doubles per particle each), radius, mass,
// fixed; a null pointer skips that array. Pointers are device memory.
struct StateIO {
  double* v[8];
  double* radius;
  double* mass;
  uint8_t* fixed;
};
// id -> slot for the `live` particles: slot_of indexed by upload position,
// then (when some were removed) compacted by a scan of the live flags into
// slot_of_id. Returns the map to use; buffers of n entries, part for the scan.
struct IdMap {
  uint32_t *slot_of, *live, *pos, *slot_of_id, *part;
};
// n_ids: upload positions (the tags range over [0, n_ids)); live: particles alive.
const uint32_t* launch_slot_of(const StepParams& P, const IdMap& M, int live, int n_ids, cudaStream_t s);
void launch_state_gather(const StepParams& P, const uint32_t* slot_of, const StateIO& io, int m, cudaStream_t s);
void launch_state_same(const StepParams& P, const uint32_t* slot_of, const StateIO& io, unsigned* differs, int m,
                       cudaStream_t s);
void launch_state_scatter(const StepParams& P, const uint32_t* slot_of, const StateIO& io, int m, cudaStream_t s);

}  // namespace rp
