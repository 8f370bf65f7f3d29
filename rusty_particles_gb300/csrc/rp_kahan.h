// The residual of one Kahan step on the integer pipe.
//
// A compensated add s += d with residual c (the reference's integrator) is
//   y = d - c;  t = s + y;  c' = (t - s) - y;  s' = t
// in FP64. On GB300 the FP64 unit runs 1/58 of the FP32 rate and the
// integrator is bound by it, while the integer pipes idle. When |s| >= |y|,
// Dekker's Fast2Sum theorem (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2) makes
// both subtractions of c' exact, so c' is the exact value t - s - y, and that
// value can be formed from the bit fields of s, y and t with integer
// arithmetic: same bits as the FP64 operations, without the FP64 unit.
//
// kahan_residual(s, y, t, c) writes c' and returns true in that case, for
// finite normal operands whose exponents lie within 60 of each other and
// whose result is normal (or zero); otherwise it returns false and leaves c
// untouched, and the caller forms c' in FP64. Plain C++ (host and device), so
// the bit-exactness can be checked on the host against FP64 hardware.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define RP_HD __host__ __device__ __forceinline__
#else
#define RP_HD inline
#endif

namespace rp {

RP_HD uint64_t f64_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof(b));
  return b;
#endif
}

RP_HD double f64_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof(x));
  return x;
#endif
}

RP_HD int clz64(uint64_t a) {  // a != 0
#if defined(__CUDA_ARCH__)
  return __clzll((long long)a);
#else
  return __builtin_clzll(a);
#endif
}

RP_HD bool kahan_residual(double s, double y, double t, double& c) {
  constexpr uint64_t kAbs = 0x7FFFFFFFFFFFFFFFull, kMant = 0x000FFFFFFFFFFFFFull, kHidden = 0x0010000000000000ull;
  const uint64_t bs = f64_bits(s), by = f64_bits(y), bt = f64_bits(t);
  if ((bs & kAbs) < (by & kAbs)) return false;  // Fast2Sum needs |s| >= |y|
  const int es = (int)((bs >> 52) & 0x7FF), ey = (int)((by >> 52) & 0x7FF), et = (int)((bt >> 52) & 0x7FF);
  // y and t normal and finite (then s, with |s| >= |y|, is normal or inf)
  if (ey == 0 || et == 0 || es == 0x7FF || et == 0x7FF) return false;
  if (es - ey > 60) return false;
  const int q = es < et ? es : et;
  if ((es > et ? es : et) - q > 1) return false;  // t within a binade of s (no deep cancellation)
  // signed significands, value = M 2^(e - 1075)
  const int64_t Ms = (int64_t)((bs & kMant) | kHidden), My = (int64_t)((by & kMant) | kHidden),
                Mt = (int64_t)((bt & kMant) | kHidden);
  const int64_t S = (bs >> 63) ? -Ms : Ms, Y = (by >> 63) ? -My : My, T = (bt >> 63) ? -Mt : Mt;
  // t - s at the scale 2^(q - 1075): |D| < 2^55
  const int64_t D = (int64_t)((uint64_t)T << (et - q)) - (int64_t)((uint64_t)S << (es - q));
  // t - s - y: |t - s| <= |y| + ulp(t)/2, so at y's scale the magnitude stays
  // below 2^53 + 2^(et - ey - 1) < 2^62
  int64_t R;
  int b;
  if (q >= ey) {
    R = (int64_t)((uint64_t)D << (q - ey)) - Y;
    b = ey;
  } else {  // q == ey - 1 (q >= es - 1 >= ey - 1)
    R = D - (int64_t)((uint64_t)Y << (ey - q));
    b = q;
  }
  if (R == 0) {  // x - x is +0 under round to nearest
    c = 0.0;
    return true;
  }
  const uint64_t neg = R < 0 ? 1ull : 0ull;
  const uint64_t A = neg ? (uint64_t)(-R) : (uint64_t)R;
  const int p = 63 - clz64(A);  // leading bit of |R|
  const int e = b + p - 52;     // biased exponent of the result
  if (e < 1 || e > 2046) return false;
  uint64_t M;
  if (p > 52) {
    if (A & ((1ull << (p - 52)) - 1ull)) return false;  // not representable (cannot happen for exact inputs)
    M = A >> (p - 52);
  } else {
    M = A << (52 - p);
  }
  c = f64_from_bits((neg << 63) | ((uint64_t)e << 52) | (M & kMant));
  return true;
}

}  // namespace rp
