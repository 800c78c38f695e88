// Exactly rounded FP64 results built with integer arithmetic (the FP64 pipe of
// this GPU retires ~2 operations per clock per SM; integer multiplies and
// shifts run far wider).  Host and device share these definitions, so the
// CPU tests check the very code the kernels run against IEEE arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#include <cmath>

#if defined(__CUDACC__)
#define A4G_HD __host__ __device__ __forceinline__
#else
#define A4G_HD inline
#endif

namespace a4g {

A4G_HD int clz64(unsigned long long x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}
A4G_HD unsigned long long mulhi64(unsigned long long a, unsigned long long b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}
A4G_HD unsigned long long bits_of(double x) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
A4G_HD double double_of(unsigned long long u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
// 1/x rounded to the nearest float
A4G_HD float frcp_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}

// The double nearest (ties to even) to u * 2^e2 with sign `neg`, u an
// unsigned 64-bit magnitude.  Results outside the normal range take an FP64
// path (ldexp).
A4G_HD double u64_scaled_to_double(unsigned long long u, bool neg, int e2) {
  if (u == 0) return 0.0;
  const int nbits = 64 - clz64(u);
  unsigned long long mant;
  int e = e2;
  if (nbits <= 53) {
    mant = u << (53 - nbits);
    e -= 53 - nbits;
  } else {
    const int sh = nbits - 53;
    mant = u >> sh;
    const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    e += sh;
    if (mant == (1ull << 53)) mant >>= 1, ++e;
  }
  const int field = e + 52 + 1023;  // value = mant * 2^e, mant in [2^52, 2^53)
  if (field >= 1 && field <= 2046)
    return double_of((neg ? (1ull << 63) : 0ull) | ((unsigned long long)field << 52) | (mant & ((1ull << 52) - 1)));
  const double v = ldexp(double(mant), e);
  return neg ? -v : v;
}

// (neg ? -1 : 1) * v * 2^e2 rounded once to the nearest double (ties to
// even), v a signed 64-bit integer: normalise, keep 53 bits, round on the 11
// below, and build the bits by one addition (a mantissa that rounds up to
// 2^53 carries into the exponent field).  Branch-free for results in the
// normal range; the rest takes u64_scaled_to_double.  Same bits as negating
// the result of u64_scaled_to_double (a zero keeps the sign the negation
// gives it).
A4G_HD double i64_scaled_to_double(long long v, int e2, bool neg) {
  const unsigned long long sign = (v < 0) != neg ? (1ull << 63) : 0ull;
  const unsigned long long u = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int n = clz64(u | 1ull);  // u = 0 is mapped to a signed zero at the end
  const unsigned long long norm = u << n;  // leading one at bit 63
  unsigned long long mant = norm >> 11;    // 53 bits, leading one at bit 52
  const unsigned long long rem = norm & 0x7FFull;
  mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  const int field = e2 + 63 - n + 1023;  // biased exponent of the leading one
  if (u != 0 && (field < 1 || field > 2045)) return u64_scaled_to_double(u, sign != 0, e2);
  const unsigned long long bits =
      u ? sign | ((((unsigned long long)(field - 1)) << 52) + mant) : (neg ? (1ull << 63) : 0ull);
  return double_of(bits);
}

// The same for a two's-complement 128-bit integer N.
A4G_HD double i128_scaled_to_double(__int128 N, int e2) {
  const bool neg = N < 0;
  const unsigned __int128 u = neg ? (unsigned __int128)(-N) : (unsigned __int128)N;
  const unsigned long long hi = (unsigned long long)(u >> 64);
  if (hi == 0) return u64_scaled_to_double((unsigned long long)u, neg, e2);
  // keep the top 63 bits and fold the rest into a sticky bit below them (the
  // rounding position lies above it, so the rounding is exact)
  const int sh = 65 - clz64(hi);  // u >> sh has 63 bits
  const unsigned long long top = (unsigned long long)(u >> sh);
  const bool sticky = (u & ((((unsigned __int128)1) << sh) - 1)) != 0;
  return u64_scaled_to_double((top << 1) | (sticky ? 1ull : 0ull), neg, e2 + sh - 1);
}

// a / b rounded to the nearest double (ties to even; a quotient of two
// doubles is never exactly halfway) for normal a, b and a normal result;
// false otherwise (the caller divides in FP64).  With A = ma or 2 ma (the
// dividend's significand doubled when it is below the divisor's, so that
// A / mb lies in [1, 2)), the 55-bit quotient Q = floor(A 2^54 / mb) is
// estimated through a reciprocal R ~ 2^116 / mb of the divisor's 53-bit
// significand and corrected from the exact remainder A 2^54 - Q mb (Knuth,
// TAOCP vol. 2, 4.3.1: estimate a quotient digit, then fix it from the
// remainder), which also gives the sticky bit for the rounding.  R comes from
// Newton-Raphson, x' = x + x (1 - d x), in fixed point: the FP32 reciprocal
// of mb's top 24 bits (relative error below 2^-22), one step in 32-bit
// arithmetic on mb's top 32 bits (below 2^-30), one step in 64-bit arithmetic
// on all of mb (below 2^-59).  Q is then off by at most one unit, so one
// correction each way suffices, and the remainder, below 2 mb < 2^54 in
// magnitude, is exact in wrapping 64-bit arithmetic.
A4G_HD bool div_rn_int(double a, double b, double* q) {
  const unsigned long long ua = bits_of(a), ub = bits_of(b);
  const int ea = int((ua >> 52) & 0x7FF), eb = int((ub >> 52) & 0x7FF);
  if (ea == 0 || ea == 2047 || eb == 0 || eb == 2047) return false;
  const unsigned long long ma = (ua & ((1ull << 52) - 1)) | (1ull << 52);
  const unsigned long long mb = (ub & ((1ull << 52) - 1)) | (1ull << 52);
  const int adj = ma < mb ? 1 : 0;
  const unsigned long long A = ma << adj;  // [mb, 2 mb)
  const int field = ea - eb + 1023 - adj;  // biased exponent of the quotient's leading bit
  if (field < 1 || field > 2045) return false;
  // seed R32 ~ 2^84 / mb: the FP32 reciprocal of mb's top 24 bits (exact in
  // FP32) lies in (2^-24, 2^-23]; its significand shifted into place, 2^-23
  // itself (2^32) clamped to 2^32 - 1
  const float rf = frcp_rn(float(uint32_t(mb >> 29)));
  uint32_t rb;
  memcpy(&rb, &rf, 4);
  unsigned long long R32 = ((rb >> 23) & 0xFFu) == 103u ? ((unsigned long long)((rb & 0x7FFFFFu) | 0x800000u) << 8)
                                                         : 0xFFFFFFFFull;
  // 32-bit step on m32 = mb's top 32 bits: R32 += R32 (2^63 - m32 R32) / 2^63
  {
    const unsigned long long m32 = mb >> 21;
    const unsigned long long t = m32 * R32;  // ~2^63, |2^63 - t| < 2^42
    const bool up = t < (1ull << 63);
    const unsigned long long e = up ? (1ull << 63) - t : t - (1ull << 63);
    const unsigned long long d = mulhi64(R32 << 1, e);
    R32 = up ? R32 + d : R32 - d;
    if (R32 > 0xFFFFFFFFull) R32 = 0xFFFFFFFFull;
  }
  // 64-bit step on mb: R += R (2^116 - mb R) / 2^116
  unsigned long long R = R32 << 32;
  {
    const unsigned long long plo = mb * R, phi = mulhi64(mb, R);  // mb R (117 bits)
    const unsigned long long elo = 0ull - plo, ehi = (1ull << 52) - phi - (plo != 0 ? 1ull : 0ull);  // 2^116 - mb R
    const long long e52 = (long long)((ehi << 12) | (elo >> 52));  // (2^116 - mb R) / 2^52, |.| < 2^35
    const unsigned long long d = mulhi64(R, e52 < 0 ? (unsigned long long)(-e52) : (unsigned long long)e52);
    R = e52 < 0 ? R - d : R + d;
  }
  // Q = floor(A 2^10 R / 2^64) / 2^8 ~ A 2^54 / mb, within one unit
  unsigned long long Q = mulhi64(A << 10, R) >> 8;
  long long rem = (long long)(((A & 0x3FFull) << 54) - Q * mb);  // A 2^54 - Q mb, exact: |.| < 2^55
  if (rem < 0) --Q, rem += (long long)mb;
  if (rem >= (long long)mb) ++Q, rem -= (long long)mb;
  unsigned long long mant = Q >> 2;
  const unsigned long long guard = (Q >> 1) & 1ull, sticky = (Q & 1ull) | (rem != 0 ? 1ull : 0ull);
  mant += (guard && (sticky || (mant & 1ull))) ? 1ull : 0ull;
  *q = double_of(((ua ^ ub) & (1ull << 63)) | ((((unsigned long long)(field - 1)) << 52) + mant));
  return true;
}

// a / b rounded to the nearest double: div_rn_int where it applies, the FP64
// divide otherwise (zero, subnormal or non-finite operands or results).
A4G_HD double div_rn(double a, double b) {
  double q;
  if (div_rn_int(a, b, &q)) return q;
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// x != 0 without the FP64 pipe
A4G_HD bool nonzero(double x) { return (bits_of(x) << 1) != 0ull; }

}  // namespace a4g
