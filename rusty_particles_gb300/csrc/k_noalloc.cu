// rp_cell_sort_noalloc: the reference-grid cell hash + stable radix sort for
// callers that must not allocate device memory.
//
// Who needs it: code that drives the GPU from inside a CUDA stream capture
// (cudaMalloc is not a stream operation and breaks the capture), engines that
// own all device memory through their own pool and forbid allocations behind
// their back (a game or robotics physics loop, a host language runtime that
// tracks every buffer), and real-time loops where cudaMalloc's implicit device
// synchronisation would stall a frame. They pass their own input and output
// buffers; the sort's temporaries live in one file-scope device array.
//
// The scratch array below is statically sized for NOALLOC_MAX_PARTICLES
// particles (about 4.3 MB) and is resident on every GPU that loads the library
// until the process exits. Every call shares it: calls whose work overlaps on
// the GPU (two streams, two threads) race on it and must be serialised by the
// caller. Nothing in it needs zeroing: every word a call reads was written
// earlier in that call.
#include <cstdint>
#include <cstring>
#include <mutex>

#include "engine.h"

namespace rp {

void set_error(const char* fmt, ...);

static constexpr uint32_t NOALLOC_MAX_PARTICLES = 1u << 18;
// keys A/B and values A/B, radix digit histograms (256 per 2048-key tile) and
// scan partials, each region starting on a 256-byte boundary
static constexpr size_t NA_KEYS = NOALLOC_MAX_PARTICLES;
static constexpr size_t NA_HIST = 256u * (NOALLOC_MAX_PARTICLES / 2048u) + 64u;
static constexpr size_t NA_PART = 4096u;
static constexpr size_t NA_WORDS = 4 * NA_KEYS + NA_HIST + NA_PART;

static __device__ __align__(256) uint32_t g_noalloc_scratch[NA_WORDS];

// Host-side address of g_noalloc_scratch per device. In host code the symbol
// name is only a stand-in for the device array; cudaGetSymbolAddress gives the
// address a kernel can use. Filled once per device by the first call and kept
// for the life of the process: it belongs to that device's context, so a
// process that resets the device (cudaDeviceReset) must not call the entry
// point again.
static std::mutex g_noalloc_mu;
static uint32_t* g_noalloc_ptr[256];

static int noalloc_scratch(int dev, uint32_t** out) {
  if (dev < 0 || dev >= 256) {
    set_error("device ordinal %d out of range", dev);
    return RP_E_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
      return RP_E_CUDA;
    }
    g_noalloc_ptr[dev] = (uint32_t*)p;
  }
  *out = g_noalloc_ptr[dev];
  return RP_OK;
}

// Cell of each position by the reference's grid formula (src/grid.rs:30-40):
// floor((x - origin) / h) per axis (saturating), linear index x + y*dx +
// z*dx*dy, or `ncells` when outside [0, dims) on any axis.
__global__ void k_noalloc_hash(const double* xyz, uint32_t n, double ox, double oy, double oz, double h, int dx,
                               int dy, int dz, uint32_t ncells, uint32_t* keys, uint32_t* vals, uint32_t* cell_of) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t cx = sat_i32(floor(__dsub_rn(xyz[3 * (size_t)i], ox) / h));
    const int32_t cy = sat_i32(floor(__dsub_rn(xyz[3 * (size_t)i + 1], oy) / h));
    const int32_t cz = sat_i32(floor(__dsub_rn(xyz[3 * (size_t)i + 2], oz) / h));
    uint32_t key = ncells;
    if (cx >= 0 && cy >= 0 && cz >= 0 && cx < dx && cy < dy && cz < dz)
      key = (uint32_t)cx + (uint32_t)cy * (uint32_t)dx + (uint32_t)cz * (uint32_t)dx * (uint32_t)dy;
    keys[i] = key;
    vals[i] = i;
    cell_of[i] = key == ncells ? 0xFFFFFFFFu : key;
  }
}

}  // namespace rp

extern "C" int rp_cell_sort_noalloc(const double* positions, size_t n, const double origin[3], double cell_size,
                                    const int32_t dims[3], uint32_t* cell_of, uint32_t* order, void* stream) {
  using namespace rp;
  if (n > NOALLOC_MAX_PARTICLES) {
    set_error("rp_cell_sort_noalloc handles at most %u particles (got %zu)", NOALLOC_MAX_PARTICLES, n);
    return RP_E_INVALID_ARG;
  }
  if (!origin || !dims || !(cell_size > 0.0) || (n && (!positions || !cell_of || !order))) {
    set_error("rp_cell_sort_noalloc: bad argument");
    return RP_E_INVALID_ARG;
  }
  uint64_t ncells = 1;
  for (int k = 0; k < 3; ++k) {
    if (dims[k] <= 0) {
      set_error("rp_cell_sort_noalloc: dims must be positive");
      return RP_E_INVALID_ARG;
    }
    ncells *= (uint64_t)dims[k];
  }
  if (ncells >= 0xFFFFFFFFull) {
    set_error("rp_cell_sort_noalloc: too many cells");
    return RP_E_INVALID_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("no usable CUDA device: %s", cudaGetErrorString(e));
    return RP_E_CUDA;
  }
  uint32_t* base = nullptr;
  int r = noalloc_scratch(dev, &base);
  if (r != RP_OK) return r;
  if (n == 0) return RP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t* ka = base;
  uint32_t* va = ka + NA_KEYS;
  uint32_t* kb = va + NA_KEYS;
  uint32_t* vb = kb + NA_KEYS;
  uint32_t* hist = vb + NA_KEYS;
  uint32_t* part = hist + NA_HIST;
  int bits = 1;
  while (bits < 32 && (1ull << bits) <= ncells) ++bits;
  k_noalloc_hash<<<grid_for(n, 256), 256, 0, s>>>(positions, (uint32_t)n, origin[0], origin[1], origin[2], cell_size,
                                                   dims[0], dims[1], dims[2], (uint32_t)ncells, ka, va, cell_of);
  int which = launch_radix_sort(nullptr, ka, va, kb, vb, (uint32_t)n, bits, hist, part, s);
  e = cudaMemcpyAsync(order, which ? vb : va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("rp_cell_sort_noalloc launch failed: %s", cudaGetErrorString(e));
    return RP_E_CUDA;
  }
  return RP_OK;
}
