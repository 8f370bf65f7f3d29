// Learned JKR contact radius.
//
// The reference solves the JKR overlap relation for the contact radius a by a
// clamped Newton iteration per contact (src/physics.rs:132-219):
//   f(a) = a^2/R* - sqrt(C a) - delta = 0,  C = 8 pi gamma / E*,
// starting from sqrt(R* delta) (delta > 0) or R*/2 (delta <= 0), at most 20
// steps, then returns zero force when |f(a)| > 1e-3 R*.
//
// In units of R* (u = a/R*, x = delta/R*, c = C/R*) the residual is
// g(u) - x with g(u) = u^2 - sqrt(c u), convex on u > 0, with its minimum
// -kappa c^(2/3) at u_c = (c/16)^(1/3), kappa = 16^(-1/6) - 16^(-2/3). Two
// exact certificates follow, and decide most pairs without any iteration:
//   ZERO       x < -kappa c^(2/3) - 1e-3: |f(a)| > 1e-3 R* for every a, so
//              whatever the iteration does the reference returns zero force.
//   CONVERGES  the reference's start lies on the increasing branch of g (for
//              delta > 0: sqrt(x) > u_c, i.e. xi = x/c^(2/3) > 16^(-2/3); for
//              delta <= 0: the start 1/2 lies right of the larger root, which
//              exists for xi > -kappa) so its Newton sequence converges to that
//              root, which any other accurate solver can then supply.
// Everything else (the sliver where the reference's iteration wanders) is left
// to the reference's own Newton.
//
// For CONVERGES pairs a 4-64-64-64-1 tanh network predicts
//   t = ln u - ln sqrt(max(x,0) + c^(2/3))
// from (overlap, R*, E*, gamma); two FP32 Newton steps polish the prediction,
// an FP64 residual check accepts it (relative residual <= 1e-6, else the
// reference's Newton runs) and one FP64 correction finishes it.
//
// Weights: FP32 masters for training (row-major [out][in], layout MO_*), BF16
// copies for inference on the tensor cores (mma.sync m16n8k16, FP32
// accumulation); the layer outputs stay in registers between layers.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace rp {

constexpr int MLP_IN = 4;
constexpr int MLP_H = 64;
// FP32 parameter block offsets
constexpr int MO_W1 = 0;
constexpr int MO_B1 = MO_W1 + MLP_H * MLP_IN;
constexpr int MO_W2 = MO_B1 + MLP_H;
constexpr int MO_B2 = MO_W2 + MLP_H * MLP_H;
constexpr int MO_W3 = MO_B2 + MLP_H;
constexpr int MO_B3 = MO_W3 + MLP_H * MLP_H;
constexpr int MO_W4 = MO_B3 + MLP_H;
constexpr int MO_B4 = MO_W4 + MLP_H;
constexpr int MLP_NPARAM = MO_B4 + 1;  // 8705

// Inference copy: BF16 bit patterns padded to the m16n8k16 shapes, FP32
// biases, the feature normalisation and the target scaling.
struct alignas(16) MlpInfer {
  uint16_t w1[MLP_H * 16];     // [64][16], inputs 4..15 zero
  uint16_t w2[MLP_H * MLP_H];  // [64][64]
  uint16_t w3[MLP_H * MLP_H];
  uint16_t w4[8 * MLP_H];      // [8][64], rows 1..7 zero
  float b1[MLP_H], b2[MLP_H], b3[MLP_H], b4;
  float xmean[4], xinv[4], ymean, ystd;
};

// ---------------------------------------------------------- certificates
constexpr float kJkrKappa = 0.472470394f;  // 16^(-1/6) - 16^(-2/3)
constexpr float kJkrXiNeg = -0.4525f;      // delta <= 0: xi >= this (roots merge at -kappa)
constexpr float kJkrXiPos = 0.16f;         // delta > 0: xi >= this (start passes u_c at 16^(-2/3) = 0.15749)
constexpr float kJkrXiWalk = 0.155f;       // delta > 0: xi <= this starts left of u_c (the walk below)
constexpr float kJkrCMin = 1e-6f;          // c range over which the reference's loop is known to converge
constexpr float kJkrCMax = 0.1f;           // (c <= 1/8 puts the start 1/2 right of every root)

// JKR_WALK: delta > 0 with the start sqrt(x) left of u_c. There df < 0, and
// f/df > a/2 <=> delta > -0.75 sqrt(C a), true for every a: the clamp binds
// at every step, so the reference's loop only halves a (exact in FP64) until
// the step a/2 drops below 1e-6 R* or 20 steps ran. Its end point is
// sqrt(R* delta) 2^-K in closed form.
enum : int { JKR_FALLBACK = 0, JKR_ZERO = 1, JKR_CONVERGES = 2, JKR_WALK = 3 };

__device__ __forceinline__ float jkr_c23(float c) { return exp2f(log2f(c) * (2.0f / 3.0f)); }

// x, c, c^(2/3) in FP32 from FP64 inputs; `pos` is the FP64 sign of the
// overlap (the reference's choice of start). Margins: the ZERO test carries
// 1e-5 relative slack against ~1e-6 of FP32 error; the xi thresholds sit 1.6 %
// and 4 % inside the exact bounds.
__device__ __forceinline__ int jkr_certify(float x, float c, float c23, bool pos) {
  if (!(c > 0.0f && c < 1e30f && c23 > 0.0f)) return JKR_FALLBACK;
  if (x + kJkrKappa * c23 + 1e-3f < -1e-5f * (fabsf(x) + c23 + 1e-3f)) return JKR_ZERO;
  if (!(c >= kJkrCMin && c <= kJkrCMax)) return JKR_FALLBACK;
  const float xi = x / c23;
  if (pos) return xi >= kJkrXiPos ? JKR_CONVERGES : (xi <= kJkrXiWalk ? JKR_WALK : JKR_FALLBACK);
  return xi >= kJkrXiNeg ? JKR_CONVERGES : JKR_FALLBACK;
}

// Raw network inputs for a pair: the overlap made dimensionless as
// sqrt(xi + kappa), xi = x / c^(2/3) (the contact radius has a square-root
// fold at xi = -kappa, which this straightens), then ln R*, ln E*, ln gamma.
__device__ __forceinline__ float jkr_overlap_feature(float x, float c23) {
  return sqrtf(fmaxf(x / c23 + kJkrKappa, 0.0f));
}
__device__ __forceinline__ void jkr_raw_features(float x, float c23, float rs, float es, float gamma, float f[4]) {
  f[0] = jkr_overlap_feature(x, c23);
  f[1] = logf(rs);
  f[2] = logf(es);
  f[3] = logf(gamma);
}
// Scale of the target: u = exp(t) * jkr_ubase(x, c23).
__device__ __forceinline__ float jkr_ubase(float x, float c23) { return sqrtf(fmaxf(x, 0.0f) + c23); }

// One clamped Newton step on g(u) - x in FP32 (returns u unchanged where the
// slope is not positive; the FP64 residual check then rejects the value).
__device__ __forceinline__ float jkr_newton_f32(float u, float x, float c) {
  const float s = sqrtf(c * u);
  const float g = u * u - s - x;
  const float dg = 2.0f * u - 0.5f * s / u;
  if (!(dg > 0.0f)) return u;
  float st = g / dg;
  const float lim = 0.5f * u;
  st = fminf(fmaxf(st, -lim), lim);
  return u - st;
}

// ------------------------------------------------------------ inference
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld_pair(const uint16_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

// One hidden layer on a 16-row tile: 4 k-tiles of A fragments in (64 inputs),
// 8 n-tiles of C fragments out (64 outputs), bias added. B fragments come
// straight from the row-major [out][in] weights: B[k][n] = W[n][k].
__device__ __forceinline__ void mlp_layer64(const uint16_t* w, const float* b, const uint32_t ain[4][4],
                                            float acc[8][4], int g, int tig) {
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float bl = b[nt * 8 + tig * 2], bh = b[nt * 8 + tig * 2 + 1];
    acc[nt][0] = bl;
    acc[nt][1] = bh;
    acc[nt][2] = bl;
    acc[nt][3] = bh;
    const uint16_t* wr = w + (nt * 8 + g) * MLP_H + tig * 2;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) mma_bf16(acc[nt], ain[kt], ld_pair(wr + kt * 16), ld_pair(wr + kt * 16 + 8));
  }
}

// tanh of the C fragments of n-tiles 2kt and 2kt+1 is exactly the A fragment
// of k-tile kt of the next layer (rows g and g+8; columns 2 tig, 2 tig + 1
// and the same + 8).
__device__ __forceinline__ void mlp_repack(const float acc[8][4], uint32_t aout[4][4]) {
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    aout[kt][0] = pack_bf16(tanh_fast(acc[2 * kt][0]), tanh_fast(acc[2 * kt][1]));
    aout[kt][1] = pack_bf16(tanh_fast(acc[2 * kt][2]), tanh_fast(acc[2 * kt][3]));
    aout[kt][2] = pack_bf16(tanh_fast(acc[2 * kt + 1][0]), tanh_fast(acc[2 * kt + 1][1]));
    aout[kt][3] = pack_bf16(tanh_fast(acc[2 * kt + 1][2]), tanh_fast(acc[2 * kt + 1][3]));
  }
}

// Warp-wide forward pass for 32 rows (lane L owns row L): normalised features
// in, normalised prediction out. All 32 lanes must call it together (the
// mma.sync instructions are warp-collective). M may point to shared memory.
__device__ __forceinline__ float mlp_forward_warp(const MlpInfer* M, const float f[4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  float out_tile[2] = {0.f, 0.f};
#pragma unroll 1
  for (int mt = 0; mt < 2; ++mt) {
    // layer 1: A rows mt*16+g and +8, inputs 2 tig and 2 tig + 1 (inputs 4..15 are zero)
    const int r0 = mt * 16 + g, r1 = r0 + 8;
    const float f0a = __shfl_sync(0xFFFFFFFFu, f[0], r0), f1a = __shfl_sync(0xFFFFFFFFu, f[1], r0);
    const float f2a = __shfl_sync(0xFFFFFFFFu, f[2], r0), f3a = __shfl_sync(0xFFFFFFFFu, f[3], r0);
    const float f0b = __shfl_sync(0xFFFFFFFFu, f[0], r1), f1b = __shfl_sync(0xFFFFFFFFu, f[1], r1);
    const float f2b = __shfl_sync(0xFFFFFFFFu, f[2], r1), f3b = __shfl_sync(0xFFFFFFFFu, f[3], r1);
    uint32_t a1[4] = {0u, 0u, 0u, 0u};
    if (tig == 0) {
      a1[0] = pack_bf16(f0a, f1a);
      a1[1] = pack_bf16(f0b, f1b);
    } else if (tig == 1) {
      a1[0] = pack_bf16(f2a, f3a);
      a1[1] = pack_bf16(f2b, f3b);
    }
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float bl = M->b1[nt * 8 + tig * 2], bh = M->b1[nt * 8 + tig * 2 + 1];
      acc[nt][0] = bl;
      acc[nt][1] = bh;
      acc[nt][2] = bl;
      acc[nt][3] = bh;
      const uint16_t* wr = M->w1 + (nt * 8 + g) * 16 + tig * 2;
      mma_bf16(acc[nt], a1, ld_pair(wr), ld_pair(wr + 8));
    }
    uint32_t a[4][4];
    mlp_repack(acc, a);
    mlp_layer64(M->w2, M->b2, a, acc, g, tig);
    mlp_repack(acc, a);
    mlp_layer64(M->w3, M->b3, a, acc, g, tig);
    mlp_repack(acc, a);
    float o[4] = {M->b4, 0.f, M->b4, 0.f};
    const uint16_t* wr = M->w4 + g * MLP_H + tig * 2;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) mma_bf16(o, a[kt], ld_pair(wr + kt * 16), ld_pair(wr + kt * 16 + 8));
    // output column 0 of row r (0..15) sits in lane 4 (r mod 8): o[0] for r < 8, o[2] above
    const int r = lane & 15;
    const float lo = __shfl_sync(0xFFFFFFFFu, o[0], 4 * (r & 7));
    const float hi = __shfl_sync(0xFFFFFFFFu, o[2], 4 * (r & 7));
    out_tile[mt] = r < 8 ? lo : hi;
  }
  return lane < 16 ? out_tile[0] : out_tile[1];
}

// Host/device helpers shared by the engine and the training code (k_mlp.cu).
struct JkrDomain {
  double rs_lo, rs_hi, es_lo, es_hi, gamma_lo, gamma_hi, x_lo, x_hi;
};

// Sample generation, training and inference (k_mlp.cu).
int jkr_generate_samples(const JkrDomain& D, uint64_t seed, size_t n, float* feat, float* target, float* weight,
                         double* a_ref, int32_t* iters, double* inputs, cudaStream_t s);
struct JkrTrainConfig {
  JkrDomain dom;
  uint64_t seed;
  size_t n_samples;  // power of two
  int epochs;
  int batch;         // multiple of 64
  float lr0, lr1;
  int qat_from_epoch;
  size_t n_val;
};
struct JkrTrainResult {
  float params[MLP_NPARAM];
  float norm[10];  // xmean[4], xinv[4], ymean, ystd
  float lo[4], hi[4];
  double final_loss, val_rms, val_max, train_ms;
  uint64_t n_valid, steps;
};
int jkr_train(const JkrTrainConfig& cfg, JkrTrainResult* out, cudaStream_t s);
void mlp_make_infer(const float* params, const float norm[10], MlpInfer* out);
int mlp_loss_grad(const float* params_d, const float* featn_d, const float* targetn_d, const float* weight_d,
                  size_t n, int qat, float* grad_d, double* loss_h, cudaStream_t s);
int mlp_infer_rows(const MlpInfer* m_d, const float* featn_d, size_t n, float* out_d, cudaStream_t s);

}  // namespace rp
