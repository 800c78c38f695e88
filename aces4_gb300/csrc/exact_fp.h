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
// unsigned 64-bit magnitude, rounded once: to 53 bits in the normal range, to
// a multiple of 2^-1074 below it (subnormal results and zero), to infinity
// beyond the largest double.
A4G_HD double u64_scaled_to_double(unsigned long long u, bool neg, int e2) {
  if (u == 0) return 0.0;
  const unsigned long long sbit = neg ? (1ull << 63) : 0ull;
  const int nbits = 64 - clz64(u);
  if (e2 + nbits - 1 < -1022) {  // below 2^-1022: the unit is 2^-1074
    const int sh = -1074 - e2;    // bits of u below the unit
    unsigned long long q;
    if (sh <= 0) {
      q = u << (-sh);  // exact: a multiple of the unit below 2^-1022
    } else if (sh > 64) {
      q = 0;  // below half a unit
    } else {
      q = sh == 64 ? 0ull : u >> sh;
      const unsigned long long rem = sh == 64 ? u : u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
      if (rem > half || (rem == half && (q & 1ull))) ++q;
    }
    return double_of(sbit | q);  // q = 2^52 (rounded up to the least normal) has the right bits too
  }
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
  if (field > 2046) return double_of(sbit | 0x7FF0000000000000ull);
  return double_of(sbit | ((unsigned long long)field << 52) | (mant & ((1ull << 52) - 1)));
}

// (neg ? -1 : 1) * v * 2^e2 rounded once to the nearest double (ties to
// even), v a signed 64-bit integer: normalise, keep 53 bits, round on the 11
// below, and build the bits by one addition (a mantissa that rounds up to
// 2^53 carries into the exponent field).  Branch-free for results in the
// normal range; the rest takes u64_scaled_to_double.  Same bits as negating
// the result of u64_scaled_to_double (a zero keeps the sign the negation
// gives it).
A4G_HD double i64_scaled_to_double(long long v, int e2, bool neg) {
#if defined(__CUDA_ARCH__)
  // On the GPU the integer-to-FP64 conversion rounds v once to 53 bits (to
  // nearest, ties to even), and the scaling by 2^e2 is an exact addition to
  // the exponent field while the result stays normal: the same bits as the
  // integer construction below, in three instructions.
  if (v != 0) {
    const unsigned long long b = bits_of(__ll2double_rn(v));
    const int field = int((b >> 52) & 0x7FF) + e2;
    if (field >= 1 && field <= 2046)
      return double_of((b + ((unsigned long long)(long long)e2 << 52)) ^ (neg ? (1ull << 63) : 0ull));
  }
#endif
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
// formed in two digits, each estimated through a 32-bit reciprocal
// R32 ~ 2^84 / mb and the next one taken from the exact remainder (Knuth,
// TAOCP vol. 2, 4.3.1: estimate a quotient digit, then continue from the
// remainder), and the last one corrected from the remainder, which also gives
// the sticky bit for the rounding.  R32 comes from Newton-Raphson,
// x' = x + x (1 - d x), in fixed point: the FP32 reciprocal of mb's top 24
// bits (relative error below 2^-22), one step in 32-bit arithmetic on mb's top
// 32 bits (below 2^-30).  Digit 1, q1 = (A's top 32 bits) R32 / 2^32, lies
// within (-2, 4.01) units of A 2^30 / mb, so s1 = A 2^30 - q1 mb (exact in
// wrapping 64-bit arithmetic) is below 4.01 mb in magnitude; digit 2,
// q2 = floor((s1 >> 25) R32 / 2^35), lies within one unit of s1 2^24 / mb
// (the estimate is off by less than 0.19 below and 0.07 above).  So
// Q = q1 2^24 + q2 is off by at most one unit, one correction each way
// suffices, and the remainder, below 2 mb < 2^54 in magnitude, is exact in
// wrapping 64-bit arithmetic.
A4G_HD bool div_rn_sig(unsigned long long ma, int ea, unsigned long long mb, int eb, unsigned long long sign,
                       double* q) {
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
  uint32_t R32 = ((rb >> 23) & 0xFFu) == 103u ? (((rb & 0x7FFFFFu) | 0x800000u) << 8) : 0xFFFFFFFFu;
  // 32-bit step on m32 = mb's top 32 bits: R32 += R32 (2^63 - m32 R32) / 2^63,
  // the correction formed from e's top 32 bits (|e| < 2^42: the seed is within
  // 2^-21 of 2^63 / m32)
  {
    const uint32_t m32 = uint32_t(mb >> 21);
    const unsigned long long t = (unsigned long long)m32 * R32;  // ~2^63
    const bool up = t < (1ull << 63);
    const unsigned long long e = up ? (1ull << 63) - t : t - (1ull << 63);
    const unsigned long long d = ((unsigned long long)R32 * uint32_t(e >> 10)) >> 53;
    const unsigned long long r = up ? (unsigned long long)R32 + d : (unsigned long long)R32 - d;
    R32 = r > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(r);
  }
  // digit 1: the quotient's top 31 bits; s1 = A 2^30 - q1 mb
  const uint32_t q1 = uint32_t(((unsigned long long)uint32_t(A >> 22) * R32) >> 32);
  const long long s1 = (long long)((A << 30) - (unsigned long long)q1 * mb);
  // digit 2: floor(s1 2^24 / mb), within one unit
  const long long q2 = ((s1 >> 25) * (long long)R32) >> 35;
  unsigned long long Q = ((unsigned long long)q1 << 24) + (unsigned long long)q2;
  long long rem = (long long)(((A & 0x3FFull) << 54) - Q * mb);  // A 2^54 - Q mb, exact: |.| < 2 mb
  if (rem < 0) --Q, rem += (long long)mb;
  if (rem >= (long long)mb) ++Q, rem -= (long long)mb;
  unsigned long long mant = Q >> 2;
  const unsigned long long guard = (Q >> 1) & 1ull, sticky = (Q & 1ull) | (rem != 0 ? 1ull : 0ull);
  mant += (guard && (sticky || (mant & 1ull))) ? 1ull : 0ull;
  *q = double_of((sign << 63) | ((((unsigned long long)(field - 1)) << 52) + mant));
  return true;
}

A4G_HD bool div_rn_int(double a, double b, double* q) {
  const unsigned long long ua = bits_of(a), ub = bits_of(b);
  const int ea = int((ua >> 52) & 0x7FF), eb = int((ub >> 52) & 0x7FF);
  if (ea == 0 || ea == 2047 || eb == 0 || eb == 2047) return false;
  const unsigned long long ma = (ua & ((1ull << 52) - 1)) | (1ull << 52);
  const unsigned long long mb = (ub & ((1ull << 52) - 1)) | (1ull << 52);
  return div_rn_sig(ma, ea, mb, eb, (ua ^ ub) >> 63, q);
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
