// The FP64 throughput of the current GPU, measured with CUDA events: the
// ceiling of the FP64-bound kernels of the step (the bit-exact Kahan
// integrator, the FP64 pair laws and the FP64 per-particle sums). Each thread
// runs eight independent chains of fused multiply-adds (or of additions), so
// the pipe, not the latency of one chain, sets the rate.
#include <algorithm>

#include "engine.h"

namespace rp {

void set_error(const char* fmt, ...);

template <bool FMA>
__global__ void __launch_bounds__(256) k_fp64_rate(double* sink, int iters, double m, double c) {
  double a[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) a[q] = 1.0 + 1e-3 * (threadIdx.x + 37 * q + blockIdx.x);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = FMA ? fma(a[q], m, c) : a[q] + c;
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s += a[q];
  if (s == -1.0) sink[0] = s;  // never true; keeps the chains live
}

}  // namespace rp

extern "C" int rp_measure_fp64_peak(double* fma_per_s, double* add_per_s) {
  using namespace rp;
  if (!fma_per_s || !add_per_s) {
    set_error("rp_measure_fp64_peak: null output");
    return RP_E_INVALID_ARG;
  }
  double* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc((void**)&sink, sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int blocks = sm_count() * 8, threads = 256, iters = 4096;
  const double ops = (double)blocks * threads * iters * 8.0;  // thread instructions per launch
  double best[2] = {0.0, 0.0};
  for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first launch warms up
      cudaEventRecord(e0);
      if (kind == 0) k_fp64_rate<true><<<blocks, threads>>>(sink, iters, 1.0 + 1e-12, 1e-13);
      else k_fp64_rate<false><<<blocks, threads>>>(sink, iters, 1.0, 1e-13);
      cudaEventRecord(e1);
      e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && rep > 0 && ms > 0.f) best[kind] = std::max(best[kind], ops / (ms * 1e-3));
    }
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (sink) cudaFree(sink);
  if (e != cudaSuccess) {
    set_error("FP64 rate probe failed: %s", cudaGetErrorString(e));
    return RP_E_CUDA;
  }
  *fma_per_s = best[0];
  *add_per_s = best[1];
  return RP_OK;
}
