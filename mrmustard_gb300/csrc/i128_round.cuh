// Correctly rounded conversion of a 128-bit integer times a power of two to double, with integer
// operations only (the slice-order recombination of the Ozaki contraction: the exact sum of all
// orders is formed as one 128-bit integer and rounded once).  Host and device.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

#if defined(__CUDACC__)
#define MM_HD __host__ __device__
#else
#define MM_HD
#endif

namespace mm {

MM_HD inline int clz64(unsigned long long x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

MM_HD inline double bits_to_double(unsigned long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// t * 2^s rounded to the nearest double, ties to even (one rounding).  Outside the normal range
// the 53-bit significand is scaled with ldexp (a second rounding only for subnormal results).
MM_HD inline double i128_scaled_to_double(__int128 t, int s) {
  if (t == 0) return 0.0;
  const bool neg = t < 0;
  const unsigned __int128 a = neg ? (unsigned __int128)0 - (unsigned __int128)t : (unsigned __int128)t;
  const unsigned long long hi = (unsigned long long)(a >> 64), lo = (unsigned long long)a;
  const int nb = hi ? 128 - clz64(hi) : 64 - clz64(lo);  // bits of |t|
  int drop = nb > 53 ? nb - 53 : 0;
  unsigned long long m = (unsigned long long)(a >> drop);  // < 2^53
  if (drop > 0) {
    const unsigned __int128 rest = a & (((unsigned __int128)1 << drop) - 1);
    const unsigned __int128 half = (unsigned __int128)1 << (drop - 1);
    if (rest > half || (rest == half && (m & 1ull))) {
      if (++m == (1ull << 53)) {
        m >>= 1;
        ++drop;
      }
    }
  }
  const int e = s + drop;  // value = m * 2^e, 1 <= m < 2^53
  const int k = 63 - clz64(m);
  const int ex = k + e + 1023;
  if (ex <= 0 || ex >= 2047) return neg ? -std::ldexp((double)m, e) : std::ldexp((double)m, e);
  const unsigned long long mant = (m << (52 - k)) & ((1ull << 52) - 1);
  return bits_to_double(((neg ? 1ull : 0ull) << 63) | ((unsigned long long)ex << 52) | mant);
}

}  // namespace mm
