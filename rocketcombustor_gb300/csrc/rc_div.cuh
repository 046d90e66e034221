// Correctly rounded FP64 division by a divisor whose reciprocal is known in
// advance, and comparisons done on bit patterns.
//
// Markstein's theorem (P. Markstein, "Computation of elementary functions on
// the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; proof in
// M. Cornea-Hasegan, R. Golliver, P. Markstein, "Correctness proofs outline
// for Newton-Raphson based floating-point divide and square root algorithms",
// ARITH-14, 1999): if y = RN(1/b) and q is a faithful approximation of a/b,
// the remainder r = a - b q is exactly representable (an FMA computes it
// exactly) and RN(q + r y) = RN(a/b), barring overflow and underflow.
//
// recip_of(b) gives yh = RN(1/b) and yl = RN((1 - b yh) yh); 1 - b yh is
// exact in one FMA, so yh + yl is within about 2^-105 of 1/b (relative).
// div_rn(a, b, yh, yl): q0 = RN(a yh + RN(a yl)) is within half an ulp plus
// about 2^-104 relative of a/b, hence faithful; r = a - b q0 exactly;
// q = RN(q0 + r yh) = RN(a/b).  Four dependent FP64 operations instead of a
// division.  A zero numerator gives a zero through the same operations; its
// sign, and the sign of every quotient, is set to sign(a) xor sign(b) on the
// bit pattern (for a non-zero quotient that is its sign already).  Operands
// whose exponents are outside [-400, 400] (where the intermediate results
// could leave the normal range), zero divisors, infinities and NaNs take the
// IEEE division.  The result equals a / b bit for bit.
#pragma once

namespace rc {

__device__ __forceinline__ bool div_rn_safe(double a, double b) {
  const int ea = (__double2hiint(a) >> 20) & 0x7ff, eb = (__double2hiint(b) >> 20) & 0x7ff;
  const bool za = (__double_as_longlong(a) << 1) == 0;
  return (za || (ea >= 1023 - 400 && ea <= 1023 + 400)) && eb >= 1023 - 400 && eb <= 1023 + 400;
}
struct Recip {
  double h, l;
};
__device__ __forceinline__ Recip recip_of(double b) {
  const double h = 1.0 / b;
  const double e = fma(-b, h, 1.0);
  return {h, e * h};
}
// a / b, given recip_of(b) = {yh, yl} (b finite and non-zero)
__device__ __forceinline__ double div_rn(double a, double b, double yh, double yl) {
  if (!div_rn_safe(a, b)) return a / b;
  const double q0 = fma(a, yh, a * yl);
  const double r = fma(-b, q0, a);
  const double q = fma(r, yh, q0);
  const int hi = (__double2hiint(q) & 0x7fffffff) | ((__double2hiint(a) ^ __double2hiint(b)) & (int)0x80000000);
  return __hiloint2double(hi, __double2loint(q));
}
// a / b for a divisor fixed in advance, its reciprocal pair given as r[0], r[1]
__device__ __forceinline__ double div_rn(double a, double b, const double* r) { return div_rn(a, b, r[0], r[1]); }

// x != 0.0 without an FP64 compare (NaN counts as non-zero, -0 as zero)
__device__ __forceinline__ bool nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }
// the bit pattern of a double; for non-negative doubles its integer order is
// the floating-point order
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// 0.0 + x on the integer pipe: x, except that -0 becomes +0 (every other
// value, NaN included, is unchanged by adding +0 in round-to-nearest)
__device__ __forceinline__ double plus_zero(double x) {
  return __double_as_longlong(x) == (long long)0x8000000000000000ULL ? 0.0 : x;
}
// 0.5 * x: for a normal x whose exponent field is at least 2 the product is
// x with that field less one, exactly; zeros, subnormals, the smallest
// normals, infinities and NaNs take the FP64 multiply
__device__ __forceinline__ double half_of(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - 2u < 0x7fdu) return __longlong_as_double(b - (1LL << 52));
  return 0.5 * x;
}

}  // namespace rc
