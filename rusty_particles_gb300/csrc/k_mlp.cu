// Learned JKR contact radius: training data from the reference's own Newton
// solver, hand-written forward/backward and Adam kernels, the BF16 inference
// copy, and a row-wise tensor-core inference kernel.
//
// Compiled with -fmad=false so the sample generator's Newton iteration rounds
// exactly as the oracle's (the labels are bit-identical to the reference
// algorithm in FP64).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "rp_launch.h"
#include "rp_mlp.cuh"

namespace rp {

namespace {

constexpr double kPiD = 3.14159265358979323846;
constexpr int kRowStride = MLP_NPARAM + 3;  // per-block partial row: gradient, loss, pad (multiple of 4)
constexpr int kSPB = 64;                    // samples per block in the training kernel
constexpr int kHS = MLP_H + 1;              // activation row stride (conflict-free column access)

#define CKM(x)                                  \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return (int)e_ + 1000; \
  } while (0)

// SplitMix64 (Steele, Lea, Flood 2014) as a counter-based generator.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uni(uint64_t seed, uint64_t i, int k) {
  return (double)(mix64(seed ^ mix64(i * 8ull + (uint64_t)k)) >> 11) * (1.0 / 9007199254740992.0);
}

// The reference's Newton iteration for the contact radius
// (src/physics.rs:164-191), in FP64 with the same operation order as the
// step kernels' JKR law; also returns how many loop bodies ran.
__device__ double jkr_reference_radius(double overlap, double es, double rs, double gamma, int* iters) {
  const double eight_pi = 8.0 * kPiD;
  const double c_val = eight_pi * gamma / es;
  const double sqrt_c = sqrt(c_val);
  double a = overlap > 0.0 ? sqrt(rs * overlap) : rs * 0.5;
  int it = 0;
  while (it < 20) {
    ++it;
    if (a <= 0.0) a = 1e-9;
    const double ts = sqrt(c_val * a);
    const double f_val = a * a / rs - ts - overlap;
    const double df = 2.0 * a / rs - 0.5 * sqrt_c / sqrt(a);
    if (fabs(df) < 1e-9) break;
    const double da = f_val / df;
    const double max_step = a * 0.5;
    double step = da;
    if (step < -max_step) step = -max_step;
    if (step > max_step) step = max_step;
    a = a - step;
    if (fabs(step) < 1e-6 * rs) break;
  }
  *iters = it;
  return a;
}

// Samples (overlap, R*, E*, gamma) over the domain: R*, E*, gamma log-uniform;
// odd samples take overlap/R* uniform over [x_lo, x_hi], even ones xi =
// x/c^(2/3) uniform over [kJkrXiNeg, min(12, x_hi / c^(2/3))] (the region
// where the contact radius varies fastest). Pairs the certificates do not
// send to the network get weight 0.
__global__ void k_jkr_samples(JkrDomain D, uint64_t seed, size_t n, float* feat, float* target, float* weight,
                              double* a_ref, int32_t* iters, double* inputs) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double rs = exp(log(D.rs_lo) + (log(D.rs_hi) - log(D.rs_lo)) * uni(seed, i, 0));
    const double es = exp(log(D.es_lo) + (log(D.es_hi) - log(D.es_lo)) * uni(seed, i, 1));
    const double gamma = exp(log(D.gamma_lo) + (log(D.gamma_hi) - log(D.gamma_lo)) * uni(seed, i, 2));
    const double C = 8.0 * kPiD * gamma / es;
    const float rsf = (float)rs;
    const float c = (float)C / rsf;
    const float c23 = jkr_c23(c);
    double x;
    if (i & 1) {
      x = D.x_lo + (D.x_hi - D.x_lo) * uni(seed, i, 3);
    } else {
      const double xhi = fmin(12.0, D.x_hi / (double)c23);
      const double xi = (double)kJkrXiNeg + (xhi - (double)kJkrXiNeg) * uni(seed, i, 3);
      x = fmax(xi * (double)c23, D.x_lo);
    }
    const double overlap = x * rs;
    const float xf = (float)overlap / rsf;
    const int cls = jkr_certify(xf, c, c23, overlap > 0.0);
    float f[4];
    jkr_raw_features(xf, c23, rsf, (float)es, (float)gamma, f);
    feat[4 * i] = f[0];
    feat[4 * i + 1] = f[1];
    feat[4 * i + 2] = f[2];
    feat[4 * i + 3] = f[3];
    int it = 0;
    double a = 0.0;
    if (cls == JKR_CONVERGES) {
      a = jkr_reference_radius(overlap, es, rs, gamma, &it);
      target[i] = (float)(log(a / rs) - log((double)jkr_ubase(xf, c23)));
      weight[i] = 1.0f;
    } else {
      target[i] = 0.0f;
      weight[i] = 0.0f;
      if (a_ref) a = jkr_reference_radius(overlap, es, rs, gamma, &it);
    }
    if (a_ref) a_ref[i] = a;
    if (inputs) {
      inputs[4 * i] = overlap;
      inputs[4 * i + 1] = rs;
      inputs[4 * i + 2] = es;
      inputs[4 * i + 3] = gamma;
    }
    if (iters) iters[i] = cls == JKR_CONVERGES ? it : -it - 100 * cls;
  }
}

__global__ void k_mlp_normalize(const float* feat, const float* target, size_t n, const float* norm, float* featn,
                                float* targetn) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 4; ++k) featn[4 * i + k] = (feat[4 * i + k] - norm[k]) * norm[4 + k];
    targetn[i] = (target[i] - norm[8]) / norm[9];
  }
}

__device__ __forceinline__ float bfr(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// Forward and backward pass of one 64-sample tile; writes the tile's summed
// gradient and loss to its partial row. Sample k of the batch is
// (a * (start + k) + b) mod n (n a power of two, a odd): a fresh permutation
// per epoch. Loss = sum_s w_s (y_s - t_s)^2 / batch. With qat the forward
// pass uses what inference uses (BF16 weights and layer inputs, tanh.approx)
// and the gradient passes the rounding straight through.
__global__ void __launch_bounds__(256) k_mlp_fwd_bwd(const float* __restrict__ params, const float* __restrict__ featn,
                                                     const float* __restrict__ targetn,
                                                     const float* __restrict__ weight, size_t n, uint64_t perm_a,
                                                     uint64_t perm_b, uint64_t start, int batch, int qat,
                                                     float* __restrict__ partial) {
  extern __shared__ float sm[];
  float* W = sm;                     // MLP_NPARAM (rounded to BF16 when qat)
  float* X = W + MLP_NPARAM + 3;     // [64][4]
  float* H1 = X + kSPB * 4;          // [64][65]
  float* H2 = H1 + kSPB * kHS;
  float* H3 = H2 + kSPB * kHS;
  float* DA = H3 + kSPB * kHS;
  float* DB = DA + kSPB * kHS;
  float* Y = DB + kSPB * kHS;        // [64] dL/dy
  float* red = Y + kSPB;             // [8]
  const int t = threadIdx.x;
  for (int p = t; p < MLP_NPARAM; p += 256) {
    const float v = params[p];
    const bool is_w = (p < MO_B1) || (p >= MO_W2 && p < MO_B2) || (p >= MO_W3 && p < MO_B3) || (p >= MO_W4 && p < MO_B4);
    W[p] = (qat && is_w) ? bfr(v) : v;
  }
  const size_t mask = n - 1;
  const uint64_t base = start + (uint64_t)blockIdx.x * kSPB;
  for (int q = t; q < kSPB * 4; q += 256) {
    const int s = q >> 2, k = q & 3;
    const size_t idx = (size_t)((perm_a * (base + s) + perm_b) & mask);
    const float v = featn[4 * idx + k];
    X[q] = qat ? bfr(v) : v;
  }
  __syncthreads();
  auto act = [&](float z) { return qat ? tanh_fast(z) : tanhf(z); };
  auto q_in = [&](float h) { return qat ? bfr(h) : h; };
  const int s_own = t & 63, g4 = t >> 6;
  // forward
  for (int r = 0; r < 16; ++r) {
    const int j = g4 + 4 * r;
    float z = W[MO_B1 + j];
#pragma unroll
    for (int k = 0; k < 4; ++k) z += W[MO_W1 + j * 4 + k] * X[s_own * 4 + k];
    H1[s_own * kHS + j] = act(z);
  }
  __syncthreads();
  for (int r = 0; r < 16; ++r) {
    const int j = g4 + 4 * r;
    float z = W[MO_B2 + j];
    for (int k = 0; k < MLP_H; ++k) z += W[MO_W2 + j * MLP_H + k] * q_in(H1[s_own * kHS + k]);
    H2[s_own * kHS + j] = act(z);
  }
  __syncthreads();
  for (int r = 0; r < 16; ++r) {
    const int j = g4 + 4 * r;
    float z = W[MO_B3 + j];
    for (int k = 0; k < MLP_H; ++k) z += W[MO_W3 + j * MLP_H + k] * q_in(H2[s_own * kHS + k]);
    H3[s_own * kHS + j] = act(z);
  }
  __syncthreads();
  float lsum = 0.f;
  if (t < kSPB) {
    float y = W[MO_B4];
    for (int k = 0; k < MLP_H; ++k) y += W[MO_W4 + k] * q_in(H3[t * kHS + k]);
    const size_t idx = (size_t)((perm_a * (base + t) + perm_b) & mask);
    const float w = weight[idx];
    const float e = y - targetn[idx];
    lsum = w * e * e;
    Y[t] = 2.0f * w * e / (float)batch;
  }
  __syncthreads();
  float* out = partial + (size_t)blockIdx.x * kRowStride;
  // output layer gradient and delta3
  if (t < MLP_H) {
    float gw = 0.f;
    for (int s = 0; s < kSPB; ++s) gw += Y[s] * q_in(H3[s * kHS + t]);
    out[MO_W4 + t] = gw;
  }
  if (t == 0) {
    float gb = 0.f;
    for (int s = 0; s < kSPB; ++s) gb += Y[s];
    out[MO_B4] = gb;
  }
  for (int r = 0; r < 16; ++r) {
    const int j = g4 + 4 * r;
    const float h = H3[s_own * kHS + j];
    DA[s_own * kHS + j] = Y[s_own] * W[MO_W4 + j] * (1.0f - h * h);
  }
  __syncthreads();
  // hidden layers 3 and 2: dW = sum_s delta (x) input, then the next delta
  auto hidden = [&](float* Dl, const float* Hin, float* Dn, int ow, int ob, bool next) {
    const int k_own = t & 63;
    for (int r = 0; r < 16; ++r) {
      const int j = g4 + 4 * r;
      float gw = 0.f;
      for (int s = 0; s < kSPB; ++s) gw += Dl[s * kHS + j] * q_in(Hin[s * kHS + k_own]);
      out[ow + j * MLP_H + k_own] = gw;
    }
    if (t < MLP_H) {
      float gb = 0.f;
      for (int s = 0; s < kSPB; ++s) gb += Dl[s * kHS + t];
      out[ob + t] = gb;
    }
    if (next) {
      for (int r = 0; r < 16; ++r) {
        const int k = g4 + 4 * r;
        float d = 0.f;
        for (int j = 0; j < MLP_H; ++j) d += Dl[s_own * kHS + j] * W[ow + j * MLP_H + k];
        const float h = Hin[s_own * kHS + k];
        Dn[s_own * kHS + k] = d * (1.0f - h * h);
      }
    }
    __syncthreads();
  };
  hidden(DA, H2, DB, MO_W3, MO_B3, true);
  hidden(DB, H1, DA, MO_W2, MO_B2, true);
  // first layer
  {
    const int j = t >> 2, k = t & 3;
    float gw = 0.f;
    for (int s = 0; s < kSPB; ++s) gw += DA[s * kHS + j] * X[s * 4 + k];
    out[MO_W1 + j * 4 + k] = gw;
    if (t < MLP_H) {
      float gb = 0.f;
      for (int s = 0; s < kSPB; ++s) gb += DA[s * kHS + t];
      out[MO_B1 + t] = gb;
    }
  }
  // tile loss
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, o);
  if ((t & 31) == 0) red[t >> 5] = lsum;
  __syncthreads();
  if (t == 0) {
    float L = 0.f;
    for (int w = 0; w < 8; ++w) L += red[w];
    out[MLP_NPARAM] = L / (float)batch;
  }
}

struct AdamArgs {
  float lr, b1, b2, eps, c1, c2;  // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)
  int update;
};

// Sums the tiles' partial rows in tile order (deterministic) and applies Adam.
__global__ void k_mlp_reduce_adam(const float* __restrict__ partial, int ntiles, float* params, float* m, float* v,
                                  float* grad_out, float* loss_out, AdamArgs A) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > MLP_NPARAM) return;
  float g = 0.f;
  for (int b = 0; b < ntiles; ++b) g += partial[(size_t)b * kRowStride + p];
  if (p == MLP_NPARAM) {
    if (loss_out) *loss_out = g;
    return;
  }
  if (grad_out) grad_out[p] = g;
  if (A.update) {
    const float mm = A.b1 * m[p] + (1.0f - A.b1) * g;
    const float vv = A.b2 * v[p] + (1.0f - A.b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    params[p] -= A.lr * (mm * A.c1) / (sqrtf(vv * A.c2) + A.eps);
  }
}

// Tensor-core inference over rows of normalised features (one row per lane).
__global__ void __launch_bounds__(128) k_mlp_infer_rows(const MlpInfer* __restrict__ Mg, const float* __restrict__ featn,
                                                        size_t n, float* __restrict__ out) {
  __shared__ MlpInfer M;
  {
    const uint4* src = reinterpret_cast<const uint4*>(Mg);
    uint4* dst = reinterpret_cast<uint4*>(&M);
    for (int i = threadIdx.x; i < (int)(sizeof(MlpInfer) / 16); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t base = ((size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < n; base += warps * 32) {
    const size_t i = base + lane;
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    if (i < n) {
#pragma unroll
      for (int k = 0; k < 4; ++k) f[k] = featn[4 * i + k];
    }
    const float y = mlp_forward_warp(&M, f);
    if (i < n) out[i] = y;
  }
}

int grid_of(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  return (int)std::max<size_t>(1, std::min<size_t>(g, (size_t)sm_count() * 32));
}

// Round-to-nearest-even FP32 -> BF16 bit pattern (NaN kept quiet).
uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7FFFFFFFu) > 0x7F800000u) return 0x7FC0;
  const uint32_t r = 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)((u + r) >> 16);
}

}  // namespace

void mlp_make_infer(const float* P, const float norm[10], MlpInfer* M) {
  std::memset(M, 0, sizeof(MlpInfer));
  for (int j = 0; j < MLP_H; ++j) {
    for (int k = 0; k < 4; ++k) M->w1[j * 16 + k] = bf16_bits(P[MO_W1 + j * 4 + k]);
    for (int k = 0; k < MLP_H; ++k) {
      M->w2[j * MLP_H + k] = bf16_bits(P[MO_W2 + j * MLP_H + k]);
      M->w3[j * MLP_H + k] = bf16_bits(P[MO_W3 + j * MLP_H + k]);
    }
    M->w4[j] = bf16_bits(P[MO_W4 + j]);
    M->b1[j] = P[MO_B1 + j];
    M->b2[j] = P[MO_B2 + j];
    M->b3[j] = P[MO_B3 + j];
  }
  M->b4 = P[MO_B4];
  for (int k = 0; k < 4; ++k) {
    M->xmean[k] = norm[k];
    M->xinv[k] = norm[4 + k];
  }
  M->ymean = norm[8];
  M->ystd = norm[9];
}

int jkr_generate_samples(const JkrDomain& D, uint64_t seed, size_t n, float* feat, float* target, float* weight,
                         double* a_ref, int32_t* iters, double* inputs, cudaStream_t s) {
  if (n == 0) return 0;
  k_jkr_samples<<<grid_of(n, 256), 256, 0, s>>>(D, seed, n, feat, target, weight, a_ref, iters, inputs);
  CKM(cudaGetLastError());
  return 0;
}

static size_t fwd_bwd_smem() {
  return sizeof(float) * ((MLP_NPARAM + 3) + kSPB * 4 + 5 * kSPB * kHS + kSPB + 8);
}

int mlp_loss_grad(const float* params_d, const float* featn_d, const float* targetn_d, const float* weight_d,
                  size_t n, int qat, float* grad_d, double* loss_h, cudaStream_t s) {
  // n must be a power of two and a multiple of 64 (identity permutation)
  if (n < kSPB || (n & (n - 1)) != 0) return -1;
  const int tiles = (int)(n / kSPB);
  float* partial = nullptr;
  float* loss_d = nullptr;
  CKM(cudaMalloc(&partial, sizeof(float) * (size_t)tiles * kRowStride));
  CKM(cudaMalloc(&loss_d, sizeof(float)));
  const size_t sm = fwd_bwd_smem();
  CKM(cudaFuncSetAttribute(k_mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  k_mlp_fwd_bwd<<<tiles, 256, sm, s>>>(params_d, featn_d, targetn_d, weight_d, n, 1, 0, 0, (int)n, qat, partial);
  AdamArgs A{};
  k_mlp_reduce_adam<<<(MLP_NPARAM + 256) / 256, 256, 0, s>>>(partial, tiles, nullptr, nullptr, nullptr, grad_d, loss_d,
                                                             A);
  float lh = 0.f;
  CKM(cudaMemcpyAsync(&lh, loss_d, sizeof(float), cudaMemcpyDeviceToHost, s));
  CKM(cudaStreamSynchronize(s));
  *loss_h = lh;
  cudaFree(partial);
  cudaFree(loss_d);
  CKM(cudaGetLastError());
  return 0;
}

int mlp_infer_rows(const MlpInfer* m_d, const float* featn_d, size_t n, float* out_d, cudaStream_t s) {
  if (n == 0) return 0;
  k_mlp_infer_rows<<<grid_of((n + 3) / 4, 32), 128, 0, s>>>(m_d, featn_d, n, out_d);
  CKM(cudaGetLastError());
  return 0;
}

// Generates the samples, normalises them, trains with Adam (cosine learning
// rate from lr0 to lr1, quantisation-aware from qat_from_epoch on) and
// measures the BF16 network on a held-out sample set.
int jkr_train(const JkrTrainConfig& cfg, JkrTrainResult* R, cudaStream_t s) {
  const size_t n = cfg.n_samples;
  if (n < 1024 || (n & (n - 1)) != 0 || cfg.batch < kSPB || cfg.batch % kSPB != 0 || (size_t)cfg.batch > n) return -1;
  const auto t0 = std::chrono::steady_clock::now();
  const size_t nv = std::max<size_t>(cfg.n_val, 1024);
  float *feat, *target, *weight, *featn, *targetn, *normd;
  float *vfeat, *vtarget, *vweight, *vfeatn, *vtargetn, *vout;
  CKM(cudaMalloc(&feat, sizeof(float) * 4 * n));
  CKM(cudaMalloc(&target, sizeof(float) * n));
  CKM(cudaMalloc(&weight, sizeof(float) * n));
  CKM(cudaMalloc(&featn, sizeof(float) * 4 * n));
  CKM(cudaMalloc(&targetn, sizeof(float) * n));
  CKM(cudaMalloc(&normd, sizeof(float) * 10));
  CKM(cudaMalloc(&vfeat, sizeof(float) * 4 * nv));
  CKM(cudaMalloc(&vtarget, sizeof(float) * nv));
  CKM(cudaMalloc(&vweight, sizeof(float) * nv));
  CKM(cudaMalloc(&vfeatn, sizeof(float) * 4 * nv));
  CKM(cudaMalloc(&vtargetn, sizeof(float) * nv));
  CKM(cudaMalloc(&vout, sizeof(float) * nv));
  int rc = jkr_generate_samples(cfg.dom, cfg.seed, n, feat, target, weight, nullptr, nullptr, nullptr, s);
  if (rc) return rc;
  rc = jkr_generate_samples(cfg.dom, cfg.seed ^ 0x5EEDF00Dull, nv, vfeat, vtarget, vweight, nullptr, nullptr, nullptr, s);
  if (rc) return rc;
  // normalisation and domain from the training set (host)
  std::vector<float> hf(4 * n), ht(n), hw(n);
  CKM(cudaMemcpyAsync(hf.data(), feat, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, s));
  CKM(cudaMemcpyAsync(ht.data(), target, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  CKM(cudaMemcpyAsync(hw.data(), weight, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  CKM(cudaStreamSynchronize(s));
  double sum[5] = {0, 0, 0, 0, 0}, sq[5] = {0, 0, 0, 0, 0};
  uint64_t nvalid = 0;
  for (int k = 0; k < 4; ++k) {
    R->lo[k] = 3e38f;
    R->hi[k] = -3e38f;
  }
  for (size_t i = 0; i < n; ++i) {
    if (hw[i] <= 0.f) continue;
    ++nvalid;
    for (int k = 0; k < 4; ++k) {
      const double v = hf[4 * i + k];
      sum[k] += v;
      sq[k] += v * v;
      R->lo[k] = std::min(R->lo[k], hf[4 * i + k]);
      R->hi[k] = std::max(R->hi[k], hf[4 * i + k]);
    }
    sum[4] += ht[i];
    sq[4] += (double)ht[i] * ht[i];
  }
  if (nvalid < 64) return -2;
  for (int k = 0; k < 5; ++k) {
    const double mu = sum[k] / nvalid;
    const double var = std::max(0.0, sq[k] / nvalid - mu * mu);
    const double sd = std::sqrt(var);
    if (k < 4) {
      R->norm[k] = (float)mu;
      R->norm[4 + k] = sd > 1e-6 ? (float)(1.0 / sd) : 0.0f;
    } else {
      R->norm[8] = (float)mu;
      R->norm[9] = sd > 1e-9 ? (float)sd : 1.0f;
    }
  }
  R->n_valid = nvalid;
  CKM(cudaMemcpyAsync(normd, R->norm, sizeof(float) * 10, cudaMemcpyHostToDevice, s));
  k_mlp_normalize<<<grid_of(n, 256), 256, 0, s>>>(feat, target, n, normd, featn, targetn);
  k_mlp_normalize<<<grid_of(nv, 256), 256, 0, s>>>(vfeat, vtarget, nv, normd, vfeatn, vtargetn);
  // parameters: uniform(-sqrt(6/(fan_in+fan_out)), +) from a hash of the seed, zero biases
  std::vector<float> P(MLP_NPARAM, 0.0f);
  auto init = [&](int off, int fo, int fi) {
    const double lim = std::sqrt(6.0 / (fi + fo));
    for (int q = 0; q < fo * fi; ++q) {
      const double u = (double)(mix64(cfg.seed * 0x100000001B3ull + (uint64_t)(off + q)) >> 11) / 9007199254740992.0;
      P[off + q] = (float)((2.0 * u - 1.0) * lim);
    }
  };
  init(MO_W1, MLP_H, MLP_IN);
  init(MO_W2, MLP_H, MLP_H);
  init(MO_W3, MLP_H, MLP_H);
  init(MO_W4, 1, MLP_H);
  float *pd, *md, *vd, *partial, *lossd;
  CKM(cudaMalloc(&pd, sizeof(float) * MLP_NPARAM));
  CKM(cudaMalloc(&md, sizeof(float) * MLP_NPARAM));
  CKM(cudaMalloc(&vd, sizeof(float) * MLP_NPARAM));
  const int tiles = cfg.batch / kSPB;
  CKM(cudaMalloc(&partial, sizeof(float) * (size_t)tiles * kRowStride));
  CKM(cudaMalloc(&lossd, sizeof(float)));
  CKM(cudaMemcpyAsync(pd, P.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, s));
  CKM(cudaMemsetAsync(md, 0, sizeof(float) * MLP_NPARAM, s));
  CKM(cudaMemsetAsync(vd, 0, sizeof(float) * MLP_NPARAM, s));
  const size_t sm = fwd_bwd_smem();
  CKM(cudaFuncSetAttribute(k_mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const uint64_t steps_per_epoch = n / (size_t)cfg.batch;
  const uint64_t total = steps_per_epoch * (uint64_t)cfg.epochs;
  double b1t = 1.0, b2t = 1.0;
  uint64_t step = 0;
  for (int ep = 0; ep < cfg.epochs; ++ep) {
    const uint64_t pa = (mix64(cfg.seed + 977ull * ep) | 1ull);
    const uint64_t pb = mix64(cfg.seed ^ (31337ull + ep));
    const int qat = ep >= cfg.qat_from_epoch ? 1 : 0;
    for (uint64_t k = 0; k < steps_per_epoch; ++k, ++step) {
      const double frac = (double)step / (double)std::max<uint64_t>(total - 1, 1);
      AdamArgs A;
      A.lr = (float)(cfg.lr1 + 0.5 * (cfg.lr0 - cfg.lr1) * (1.0 + std::cos(kPiD * frac)));
      A.b1 = 0.9f;
      A.b2 = 0.999f;
      A.eps = 1e-8f;
      b1t *= 0.9;
      b2t *= 0.999;
      A.c1 = (float)(1.0 / (1.0 - b1t));
      A.c2 = (float)(1.0 / (1.0 - b2t));
      A.update = 1;
      k_mlp_fwd_bwd<<<tiles, 256, sm, s>>>(pd, featn, targetn, weight, n, pa, pb, k * (uint64_t)cfg.batch, cfg.batch,
                                           qat, partial);
      k_mlp_reduce_adam<<<(MLP_NPARAM + 256) / 256, 256, 0, s>>>(partial, tiles, pd, md, vd, nullptr, lossd, A);
    }
  }
  CKM(cudaGetLastError());
  float lh = 0.f;
  CKM(cudaMemcpyAsync(&lh, lossd, sizeof(float), cudaMemcpyDeviceToHost, s));
  CKM(cudaMemcpyAsync(R->params, pd, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, s));
  CKM(cudaStreamSynchronize(s));
  R->final_loss = lh;
  R->steps = step;
  // held-out error of the BF16 tensor-core network, in the target t
  MlpInfer hm;
  mlp_make_infer(R->params, R->norm, &hm);
  MlpInfer* mdev = nullptr;
  CKM(cudaMalloc(&mdev, sizeof(MlpInfer)));
  CKM(cudaMemcpyAsync(mdev, &hm, sizeof(MlpInfer), cudaMemcpyHostToDevice, s));
  rc = mlp_infer_rows(mdev, vfeatn, nv, vout, s);
  if (rc) return rc;
  std::vector<float> yo(nv), yt(nv), yw(nv);
  CKM(cudaMemcpyAsync(yo.data(), vout, sizeof(float) * nv, cudaMemcpyDeviceToHost, s));
  CKM(cudaMemcpyAsync(yt.data(), vtarget, sizeof(float) * nv, cudaMemcpyDeviceToHost, s));
  CKM(cudaMemcpyAsync(yw.data(), vweight, sizeof(float) * nv, cudaMemcpyDeviceToHost, s));
  CKM(cudaStreamSynchronize(s));
  double se = 0.0, mx = 0.0;
  uint64_t cnt = 0;
  for (size_t i = 0; i < nv; ++i) {
    if (yw[i] <= 0.f) continue;
    const double e = std::fabs((double)yo[i] * R->norm[9] + R->norm[8] - (double)yt[i]);
    se += e * e;
    mx = std::max(mx, e);
    ++cnt;
  }
  R->val_rms = cnt ? std::sqrt(se / cnt) : 0.0;
  R->val_max = mx;
  for (void* p : {(void*)feat, (void*)target, (void*)weight, (void*)featn, (void*)targetn, (void*)normd, (void*)vfeat,
                  (void*)vtarget, (void*)vweight, (void*)vfeatn, (void*)vtargetn, (void*)vout, (void*)pd, (void*)md,
                  (void*)vd, (void*)partial, (void*)lossd, (void*)mdev})
    cudaFree(p);
  R->train_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  CKM(cudaGetLastError());
  return 0;
}

}  // namespace rp
