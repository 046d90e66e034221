// Portable FP64 exp, log and pow with identical results on the host (C++) and
// on the GPU (CUDA).
//
// The reference evaluates exp/log/pow through the host libm.  Two libms
// (glibc on the CPU, the CUDA math library on the GPU) differ by an ulp here
// and there, and the steady iteration can amplify such differences: the
// explicit, clipped chemical source of a nearly depleted species multiplies
// them at every iteration.  Every FP64 hot-path evaluation of exp/log/pow, on
// the CPU and on the GPU, therefore goes through these functions.  They use
// only IEEE-754 +, -, *, /, rint and explicitly fused multiply-adds (correctly
// rounded on both sides: std::fma / __fma_rn), so one input gives one output
// everywhere; the results are within a few ulp of the correctly rounded values
// (tests/test_math.py checks them against the host libm).
//
// Methods (textbook, restated here):
//   exp(x): x = k ln2 + r with k = rint(x/ln2) and r from a two-constant
//           (Cody-Waite) reduction done with FMAs, |r| <= ln2/2; exp(r) by the
//           Taylor series to r^13 in Horner form; times 2^k by exponent
//           construction.
//   log(x): x = 2^e m with m in [sqrt(2)/2, sqrt(2)), f = m - 1 exact,
//           s = f/(2+f); log(1+f) = 2 atanh(s) = f - s (f - T(s^2)) with
//           T(z) = sum_{k>=1} 2 z^k/(2k+1) (11 terms); plus e ln2.
//   pow(x,y), x > 0: exp(y log x) with the rounding error of y*log(x) carried
//           to first order.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define RCM_HD __host__ __device__ __forceinline__
#else
#define RCM_HD inline
#endif

namespace rcm {

RCM_HD double fma_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
RCM_HD double rint_(double x) {
#ifdef __CUDA_ARCH__
  return rint(x);
#else
  return std::nearbyint(x);
#endif
}
RCM_HD int64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
RCM_HD double from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// ln 2 = LN2 + LN2_TAIL (LN2 is ln 2 rounded to double)
constexpr double LN2 = 0.6931471805599453094;
constexpr double LN2_TAIL = 2.319046813846299558e-17;
constexpr double INV_LN2 = 1.4426950408889634074;

// 2^k for integer k with a normal result
RCM_HD double pow2i(int k) { return from_bits((int64_t)(k + 1023) << 52); }

// Range and special-value tests compare bit patterns (integer operations):
// for non-negative doubles the integer order of the patterns is the
// floating-point order.
constexpr int64_t ABS_MASK = 0x7fffffffffffffffLL;
constexpr int64_t INF_BITS = 0x7ff0000000000000LL;
constexpr int64_t EXP_HI_BITS = 0x40862e42fefa39efLL;  // 709.782712893384
constexpr int64_t EXP_LO_BITS = 0x40874910d52d3052LL;  // 745.1332191019412
constexpr int64_t SQRT2_BITS = 0x3ff6a09e667f3bcdLL;   // 1.4142135623730951

RCM_HD double exp(double x) {
  const int64_t b = bits(x);
  if ((b & ABS_MASK) > INF_BITS) return x;           // NaN
  if (b > EXP_HI_BITS) return HUGE_VAL;              // x > 709.782712893384
  if (b < 0 && (b & ABS_MASK) > EXP_LO_BITS) return 0.0;  // x < -745.1332191019412
  const double kd = rint_(x * INV_LN2);
  double r = fma_(-kd, LN2, x);
  r = fma_(-kd, LN2_TAIL, r);
  double p = 1.0 / 6227020800.0;               // 1/13!
  p = fma_(p, r, 1.0 / 479001600.0);           // 1/12!
  p = fma_(p, r, 1.0 / 39916800.0);            // 1/11!
  p = fma_(p, r, 1.0 / 3628800.0);             // 1/10!
  p = fma_(p, r, 1.0 / 362880.0);              // 1/9!
  p = fma_(p, r, 1.0 / 40320.0);               // 1/8!
  p = fma_(p, r, 1.0 / 5040.0);                // 1/7!
  p = fma_(p, r, 1.0 / 720.0);                 // 1/6!
  p = fma_(p, r, 1.0 / 120.0);                 // 1/5!
  p = fma_(p, r, 1.0 / 24.0);                  // 1/4!
  p = fma_(p, r, 1.0 / 6.0);                   // 1/3!
  p = fma_(p, r, 0.5);                         // 1/2!
  p = fma_(p, r, 1.0);
  p = fma_(p, r, 1.0);
  const int k = (int)kd;
  if (k >= -1021 && k <= 1023) return p * pow2i(k);
  const int k1 = k / 2;
  return (p * pow2i(k1)) * pow2i(k - k1);
}

RCM_HD double log(double x) {
  int64_t b = bits(x);
  if ((b & ABS_MASK) > INF_BITS) return x;                                    // NaN
  if (b <= 0)                                                                 // x <= 0 (incl. -0)
    return (b & ABS_MASK) == 0 ? -HUGE_VAL : (x - x) / (x - x);
  if (b == INF_BITS) return x;
  int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) {  // subnormal: scale by 2^54 (exact)
    x = x * 18014398509481984.0;
    b = bits(x);
    e = (int)((b >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  const int64_t mb = (b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL;
  double m = from_bits(mb);  // [1, 2)
  if (mb > SQRT2_BITS) {
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double z = s * s;
  double t = 2.0 / 23.0;
  t = fma_(t, z, 2.0 / 21.0);
  t = fma_(t, z, 2.0 / 19.0);
  t = fma_(t, z, 2.0 / 17.0);
  t = fma_(t, z, 2.0 / 15.0);
  t = fma_(t, z, 2.0 / 13.0);
  t = fma_(t, z, 2.0 / 11.0);
  t = fma_(t, z, 2.0 / 9.0);
  t = fma_(t, z, 2.0 / 7.0);
  t = fma_(t, z, 2.0 / 5.0);
  t = fma_(t, z, 2.0 / 3.0);
  t = t * z;
  const double lp = f - s * (f - t);
  const double ed = (double)e;
  return fma_(ed, LN2, fma_(ed, LN2_TAIL, lp));
}

// x > 0 (the reference only takes powers of positive quantities)
RCM_HD double pow(double x, double y) {
  const int64_t bx = bits(x), by = bits(y);
  if (bx == 0x3ff0000000000000LL || (by & ABS_MASK) == 0) return 1.0;  // x == 1 or y == 0
  if ((bx & ABS_MASK) == 0) return (by > 0 && (by & ABS_MASK) <= INF_BITS) ? 0.0 : HUGE_VAL;  // x == 0
  const double L = log(x);
  const double t = y * L;
  const double terr = fma_(y, L, -t);
  const double p = exp(t);
  return fma_(p, terr, p);
}

}  // namespace rcm
