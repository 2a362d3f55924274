// Exact rounding of the tensor-core update's level sums to FP64, written once for the device and the host
// (the host build is what the CPU tests check against the FP64 expression it replaces).
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#ifdef __CUDACC__
#define SKN_HD __host__ __device__ __forceinline__
#else
#define SKN_HD inline
#endif

SKN_HD int skn_clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

SKN_HD double skn_bits_to_double(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// The double nearest to (hi * 2^21 + lo) * 2^e, ties to even, assembled with integer operations: the exact
// sum is formed in 128 bits, its top 53 bits are rounded and packed with the exponent.  It equals
// fma((double)hi, 2^-35, (double)lo * 2^-56) * 2^(e + 56), one rounding of the same exact value, for
// |hi| < 2^53 and |lo| < 2^53, while keeping the int64-to-FP64 conversions and the scaling off the FP64 pipe.
// Results outside the normal range take that FP64 expression.
SKN_HD double exact_to_double(long long hi, long long lo, int e) {
  const __int128 v = ((__int128)hi << 21) + (__int128)lo;
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? 0x8000000000000000ull : 0ull;
  const unsigned __int128 a = v < 0 ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const unsigned long long ah = (unsigned long long)(a >> 64), al = (unsigned long long)a;
  int msb = ah ? 127 - skn_clz64(ah) : 63 - skn_clz64(al);   // a in [2^msb, 2^(msb+1))
  unsigned long long m;                                       // 53-bit significand
  if (msb > 52) {
    const int sh = msb - 52;
    m = (unsigned long long)(a >> sh);
    const unsigned __int128 rem = a - ((unsigned __int128)m << sh);
    const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (m & 1ull))) {
      ++m;
      if (m == (1ull << 53)) {
        m >>= 1;
        ++msb;
      }
    }
  } else {
    m = (unsigned long long)(a << (52 - msb));
  }
  const int be = msb + e + 1023;                              // value = m * 2^(msb - 52 + e), m in [2^52, 2^53)
  if (be <= 0 || be >= 2047) return fma((double)hi, 0x1p-35, (double)lo * 0x1p-56) * ldexp(1.0, e + 56);
  return skn_bits_to_double(sgn | ((unsigned long long)be << 52) | (m & 0xFFFFFFFFFFFFFull));
}
