// Host run of the library's exact-rounding helpers (the same source the
// kernels compile) against IEEE arithmetic: the division against a / b, the
// scaled integer conversions against a long double reference (64 or more
// significand bits: exact for the integers tested, one rounding to double).
#include <stdio.h>

#include <cmath>
#include <random>
#include <vector>

#include "exact_fp.h"

using namespace a4g;

static bool same(double x, double y) { return bits_of(x) == bits_of(y); }

// Reference rounding of a 128-bit magnitude times 2^e2 (normal results):
// take the top 53 bits, round half to even on all the bits below.
static double ref128(unsigned __int128 mag, bool neg, int e2) {
  int nb = 0;
  for (unsigned __int128 t = mag; t; t >>= 1) ++nb;
  unsigned long long mant;
  int e = e2;
  if (nb <= 53) {
    mant = (unsigned long long)mag;
  } else {
    const int sh = nb - 53;
    mant = (unsigned long long)(mag >> sh);
    const unsigned __int128 rem = mag & ((((unsigned __int128)1) << sh) - 1), half = ((unsigned __int128)1) << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    e += sh;
  }
  const double v = std::ldexp((double)mant, e);
  return neg ? -v : v;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 2000000;
  std::mt19937_64 g(20261204);
  long bad = 0, fast = 0;
  // division: random significands and exponents, short and all-ones significands,
  // powers of two, and denominator-like operands
  std::uniform_real_distribution<double> U(-2.0, 5.0), X(-1.0, 1.0);
  for (long i = 0; i < n; ++i) {
    unsigned long long ua = g(), ub = g();
    ua = (ua & 0x800FFFFFFFFFFFFFull) | ((unsigned long long)(900 + g() % 250) << 52);
    ub = (ub & 0x800FFFFFFFFFFFFFull) | ((unsigned long long)(900 + g() % 250) << 52);
    if (i % 5 == 1) ub &= ~((1ull << (g() % 52)) - 1);
    if (i % 5 == 2) ua &= ~((1ull << (g() % 52)) - 1);
    if (i % 7 == 3) ub &= 0xFFF0000000000000ull;
    if (i % 11 == 4) ub |= 0x000FFFFFFFFFFFFFull;
    if (i % 13 == 5) ua |= 0x000FFFFFFFFFFFFFull;
    double a = double_of(ua), b = double_of(ub);
    if (i % 3 == 0) a = X(g) * 1e-3, b = U(g) + U(g) - U(g) - U(g);
    double q;
    if (div_rn_int(a, b, &q)) {
      ++fast;
      if (!same(q, a / b)) {
        if (bad < 5) printf("div: a=%a b=%a got %a want %a\n", a, b, q, a / b);
        ++bad;
      }
    } else if (std::isnormal(a) && std::isnormal(b) && std::isnormal(a / b) && std::fabs(std::log2(std::fabs(a / b))) < 900) {
      if (bad < 5) printf("div: unexpected fallback a=%a b=%a\n", a, b);
      ++bad;
    }
  }
  // division: every pair of edge significands (the ends of [2^52, 2^53), one
  // bit set or cleared above the leading one), both orders of magnitude
  {
    std::vector<unsigned long long> sig;
    for (int k = 0; k < 4; ++k) sig.push_back((1ull << 52) + k), sig.push_back((2ull << 52) - 1 - k);
    for (int k = 0; k < 52; ++k) sig.push_back((1ull << 52) | (1ull << k)), sig.push_back(((2ull << 52) - 1) & ~(1ull << k));
    for (int k = 0; k < 40; ++k) sig.push_back((1ull << 52) | (g() >> 12));
    for (unsigned long long sa : sig)
      for (unsigned long long sb : sig)
        for (int de = -1; de <= 1; ++de) {
          const double a = double_of(((unsigned long long)(1023 + de) << 52) | (sa & ((1ull << 52) - 1)));
          const double b = double_of((1023ull << 52) | (sb & ((1ull << 52) - 1)));
          double q;
          if (!div_rn_int(a, b, &q) || !same(q, a / b)) {
            if (bad < 10) printf("div edge: a=%a b=%a\n", a, b);
            ++bad;
          }
          ++fast;
        }
  }
  // scaled integer -> double, both signs, ties and near-ties
  for (long i = 0; i < n; ++i) {
    const int bits = 1 + int(g() % 63);
    long long v = (long long)(g() >> (64 - bits));
    if (i % 4 == 1) v = (long long)((((g() >> 40) | 1ull) << (g() % 30)));  // exact / tie patterns
    if (g() & 1) v = -v;
    const int e2 = -300 + int(g() % 500);
    const bool neg = g() & 1;
    const long double r = std::ldexp((long double)v, e2);
    const double want = (double)(neg ? -r : r);
    const double got = i64_scaled_to_double(v, e2, neg);
    const double want_zero_sign = v == 0 ? (neg ? -0.0 : 0.0) : want;
    if (!same(got, want_zero_sign)) {
      if (bad < 10) printf("i64: v=%lld e2=%d neg=%d got %a want %a\n", v, e2, int(neg), got, want_zero_sign);
      ++bad;
    }
    const double got_u = u64_scaled_to_double(v < 0 ? (unsigned long long)(-v) : (unsigned long long)v, v < 0, e2);
    if (v != 0 && !same(got_u, (double)r)) {
      if (bad < 10) printf("u64: v=%lld e2=%d got %a want %a\n", v, e2, got_u, (double)r);
      ++bad;
    }
    // 128-bit: v * 2^k + low bits
    const int k = int(g() % 60);
    const unsigned long long low = k ? (g() >> (64 - k)) : 0ull;
    const __int128 N = ((__int128)v << k) + (__int128)(v < 0 ? -(long long)low : (long long)low);
    const long double rn = std::ldexp((long double)v, e2 + k) + (v < 0 ? -1.0L : 1.0L) * std::ldexp((long double)low, e2);
    const unsigned __int128 mag = N < 0 ? (unsigned __int128)(-N) : (unsigned __int128)N;
    if (mag != 0 && (mag >> 64) == 0 && !same(i128_scaled_to_double(N, e2), (double)rn)) {
      if (bad < 10) printf("i128 (64-bit range): v=%lld k=%d e2=%d\n", v, k, e2);
      ++bad;
    }
    // beyond 64 bits: the sticky-bit path against the direct rounding
    const unsigned __int128 big = (((unsigned __int128)g()) << (int(g() % 60) + 1)) ^ g();
    const bool bneg = g() & 1;
    const __int128 B = bneg ? -(__int128)big : (__int128)big;
    if (big != 0 && !same(i128_scaled_to_double(B, e2), ref128(big, bneg, e2))) {
      if (bad < 10) printf("i128: e2=%d\n", e2);
      ++bad;
    }
  }
  // scaled integer -> double at the ends of the range: subnormal results,
  // underflow to zero and overflow to infinity, rounded once
  for (long i = 0; i < n; ++i) {
    const int bits = 1 + int(g() % 63);
    long long v = (long long)(g() >> (64 - bits));
    if (g() & 1) v = -v;
    const int e2 = (i & 1) ? -1150 + int(g() % 130) : 940 + int(g() % 80);
    const bool neg = g() & 1;
    const long double r = std::ldexp((long double)v, e2);
    const double want = v == 0 ? (neg ? -0.0 : 0.0) : (double)(neg ? -r : r);
    const double got = i64_scaled_to_double(v, e2, neg);
    if (!same(got, want)) {
      if (bad < 10) printf("i64 extreme: v=%lld e2=%d neg=%d got %a want %a\n", v, e2, int(neg), got, want);
      ++bad;
    }
  }
  printf("division checked %ld on the integer path, mismatches %ld\n", fast, bad);
  return bad == 0 && fast > n / 2 ? 0 : 1;
}
