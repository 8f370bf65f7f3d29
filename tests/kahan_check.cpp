// Checks rp::kahan_residual against FP64 hardware: for t = s + y, whenever
// the integer path answers, its bits must equal those of (t - s) - y.
// Built and run by tests/test_kahan_residual.py:
//   g++ -O2 -ffp-contract=off -I rusty_particles_gb300/csrc tests/kahan_check.cpp
//   ./a.out <cases> <seed>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "rp_kahan.h"

static uint64_t state;
static uint64_t next_u64() {  // SplitMix64 (Steele, Lea, Flood 2014)
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double unit() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
static double sign() { return (next_u64() & 1) ? -1.0 : 1.0; }

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  long fast = 0, bad = 0;
  for (long i = 0; i < n; ++i) {
    double s, y;
    switch (i % 6) {
      case 0:  // magnitudes of a DEM integrator: state and small increments
        s = sign() * std::pow(10.0, -6.0 + 9.0 * unit());
        y = s * sign() * std::pow(10.0, -18.0 * unit());
        break;
      case 1: {  // increment minus a residual, as the integrator forms y
        s = sign() * std::pow(10.0, -3.0 + 4.0 * unit());
        const double d = s * sign() * std::pow(10.0, -12.0 * unit());
        const double c = d * sign() * std::pow(10.0, -16.0 - 4.0 * unit());
        y = d - c;
        break;
      }
      case 2: {  // near cancellation and exact ratios
        s = sign() * (1.0 + unit()) * std::ldexp(1.0, (int)(next_u64() % 200) - 100);
        const int k = (int)(next_u64() % 8);
        y = (k == 0) ? -s : (k == 1) ? -s * 0.5 : (k == 2) ? -std::nextafter(s, 0.0)
            : (k == 3) ? std::ldexp(s, -(int)(next_u64() % 64)) : (k == 4) ? -std::ldexp(s, -1 - (int)(next_u64() % 3))
            : s * (unit() - 0.5) * 2.0;
        break;
      }
      case 3: {  // arbitrary exponents within 70 binades
        const uint64_t e1 = 1 + next_u64() % 2046;
        const uint64_t de = next_u64() % 70;
        const uint64_t e2 = e1 > de ? e1 - de : 1;
        uint64_t b1 = (next_u64() & 0x800FFFFFFFFFFFFFull) | (e1 << 52);
        uint64_t b2 = (next_u64() & 0x800FFFFFFFFFFFFFull) | (e2 << 52);
        std::memcpy(&s, &b1, 8);
        std::memcpy(&y, &b2, 8);
        break;
      }
      case 4: {  // raw bit patterns (zeros, subnormals, inf, NaN included)
        uint64_t b1 = next_u64(), b2 = next_u64();
        if (next_u64() % 4 == 0) b2 = b1 ^ (next_u64() & 0x8000000000000FFFull);
        std::memcpy(&s, &b1, 8);
        std::memcpy(&y, &b2, 8);
        break;
      }
      default:  // tiny magnitudes near the normal range's lower end
        s = sign() * std::ldexp(1.0 + unit(), -1000 - (int)(next_u64() % 22));
        y = s * sign() * std::ldexp(unit(), -(int)(next_u64() % 40));
        break;
    }
    const double t = s + y;
    const double ref = (t - s) - y;
    double c = 12345.0;
    if (rp::kahan_residual(s, y, t, c)) {
      ++fast;
      uint64_t a, b;
      std::memcpy(&a, &c, 8);
      std::memcpy(&b, &ref, 8);
      if (a != b) {
        if (bad < 10)
          std::printf("MISMATCH s=%a y=%a t=%a int=%a fp64=%a\n", s, y, t, c, ref);
        ++bad;
      }
    }
  }
  std::printf("cases %ld fast %ld mismatches %ld\n", n, fast, bad);
  return bad ? 1 : 0;
}
