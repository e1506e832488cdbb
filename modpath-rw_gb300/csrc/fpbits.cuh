// fpbits.cuh -- FP64 tests and compares taken from IEEE-754 bit patterns on
// the integer pipe, and the Irwin-Hall normal assembled from its bits.
//
// GB300 issues two FP64 lanes per clock per SM, so an FP64 compare holds the
// FP64 pipe as long as a multiply-add; the FP64 step kernel is bound by that
// pipe.  Each function here gives the FP64 compare's answer for every input
// (signed zeros, subnormals and infinities as the compare orders them, NaN
// false like the compare) in a few integer instructions.  A range test is one
// unsigned subtraction and compare: b in [lo, hi] <=> b - lo < hi - lo + 1.
// The header also compiles as plain C++ for the host, where the tests check
// every function against the compare it replaces.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define MPRW_FB __host__ __device__ __forceinline__
#else
#define MPRW_FB inline
#endif

namespace mprw {
namespace fb {

MPRW_FB unsigned long long bits(double v) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(v);
#else
  unsigned long long b;
  std::memcpy(&b, &v, sizeof b);
  return b;
#endif
}

MPRW_FB double from_bits(unsigned long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double v;
  std::memcpy(&v, &b, sizeof v);
  return v;
#endif
}

// v > 1: bits in (bits(1), bits(+inf)]
MPRW_FB bool above1(double v) { return bits(v) - 0x3FF0000000000001ULL < 0x4000000000000000ULL; }
// v < 0: bits in (bits(-0), bits(-inf)]; -0 is not below 0
MPRW_FB bool below0(double v) { return bits(v) - 0x8000000000000001ULL < 0x7FF0000000000000ULL; }
// v > 0: bits in (bits(+0), bits(+inf)]
MPRW_FB bool above0(double v) { return bits(v) - 1ULL < 0x7FF0000000000000ULL; }
// v == 0: +0 or -0
MPRW_FB bool is0(double v) { return (bits(v) << 1) == 0ULL; }
// v == 1
MPRW_FB bool is1(double v) { return bits(v) == 0x3FF0000000000000ULL; }
// v >= 0: [+0, +inf] or -0
MPRW_FB bool nonneg(double v) {
  const unsigned long long b = bits(v);
  return (b <= 0x7FF0000000000000ULL) | (b == 0x8000000000000000ULL);
}
// |v| > 1/2: |v|'s bits in (bits(1/2), bits(+inf)]
MPRW_FB bool abs_above_half(double v) {
  return (bits(v) & 0x7FFFFFFFFFFFFFFFULL) - 0x3FE0000000000001ULL < 0x4010000000000000ULL;
}
// v > 1 or v < 0
MPRW_FB bool out01(double v) { return above1(v) | below0(v); }
// a < b for a, b > 0 (not NaN): the bit patterns of positive doubles are
// ordered as their values
MPRW_FB bool pos_lt(double a, double b) { return bits(a) < bits(b); }

// a < b and a == b for any two doubles.  Mapped to two's-complement keys
// (negative values: the magnitude bits flipped, so larger magnitudes are
// smaller keys; -0 first taken as +0) the keys are ordered as the values.
MPRW_FB bool isnan_bits(double v) { return (bits(v) & 0x7FFFFFFFFFFFFFFFULL) > 0x7FF0000000000000ULL; }
MPRW_FB long long order_key(double v) {
  long long b = (long long)bits(v);
  b = (b == (long long)0x8000000000000000ULL) ? 0LL : b;
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
MPRW_FB bool lt_any(double a, double b) {
  return !(isnan_bits(a) | isnan_bits(b)) & (order_key(a) < order_key(b));
}
MPRW_FB bool eq_any(double a, double b) {
  return !(isnan_bits(a) | isnan_bits(b)) & (order_key(a) == order_key(b));
}

// maxTime < t (the end of the tracking interval passed): for maxTime in
// [+0, +inf] exactly one unsigned range test on t's bits, t > maxTime <=>
// bits(t) in [bits(maxTime) + 1, bits(+inf)] (NaN and negative t fall
// outside); any other maxTime takes the FP64 compare.  In a kernel the branch
// is uniform (maxTime is the launch's).
MPRW_FB bool past_end(double maxTime, double t) {
  const unsigned long long km = bits(maxTime);
  if (km <= 0x7FF0000000000000ULL) return bits(t) - (km + 1ULL) < 0x7FF0000000000000ULL - km;
  return maxTime < t;
}

MPRW_FB int clz64(unsigned long long m) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)m);
#else
  return m ? __builtin_clzll(m) : 64;
#endif
}

// The Irwin-Hall(12) normal S*2^-32 - 6 of the 36-bit sum S of twelve 32-bit
// words, exact (|S - 6*2^32| < 2^36), assembled from its sign, exponent and
// mantissa: the same bits as (2^20 + S*2^-32) - (2^20 + 6) in FP64, +0 for
// S = 6*2^32.
MPRW_FB double ih12_normal(unsigned long long sum) {
  const long long k = (long long)sum - (6LL << 32);
  const unsigned long long m = (unsigned long long)(k < 0 ? -k : k);
  const int e = 63 - clz64(m);  // most significant bit, 0..35
  const unsigned long long b = ((unsigned long long)k & 0x8000000000000000ULL) |
                               ((unsigned long long)(e + 991) << 52) |  // 991 = 1023 - 32
                               ((m << (52 - e)) & 0x000FFFFFFFFFFFFFULL);
  return from_bits(m ? b : 0ULL);
}

}  // namespace fb
}  // namespace mprw
