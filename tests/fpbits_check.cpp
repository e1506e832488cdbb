// Host check of modpath-rw_gb300/csrc/fpbits.cuh: every bit-pattern test and
// compare against the IEEE-754 compare it stands for, and the Irwin-Hall
// normal against the FP64 subtraction it replaces, on special values, values
// next to each boundary and random bit patterns.  Prints "ok <n>" or the first
// mismatches; exit status 1 on a mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "fpbits.cuh"

using namespace mprw::fb;

static long long g_checked = 0, g_bad = 0;

static void expect(bool got, bool want, const char *what, double a, double b = 0.0) {
  ++g_checked;
  if (got != want && g_bad++ < 20)
    std::printf("MISMATCH %s a=%a (%016llx) b=%a got %d want %d\n", what, a, bits(a), b, (int)got, (int)want);
}

int main() {
  const double inf = std::numeric_limits<double>::infinity();
  const double qnan = std::numeric_limits<double>::quiet_NaN();
  std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, inf, -inf, qnan, -qnan,
                           std::numeric_limits<double>::denorm_min(), -std::numeric_limits<double>::denorm_min(),
                           std::numeric_limits<double>::min(), -std::numeric_limits<double>::min(),
                           std::numeric_limits<double>::max(), -std::numeric_limits<double>::max(), 130.0, 1e-300};
  for (double c : {0.0, 0.5, 1.0, -0.5, -1.0, 130.0})
    for (double d : {inf, -inf}) {
      double x = c;
      for (int i = 0; i < 4; ++i) {
        x = std::nextafter(x, d);
        v.push_back(x);
      }
    }
  for (unsigned long long nb : {0x7FF0000000000001ULL, 0xFFF0000000000001ULL, 0x7FF8000000000000ULL,
                                0x7FFFFFFFFFFFFFFFULL, 0xFFFFFFFFFFFFFFFFULL, 0x8000000000000001ULL})
    v.push_back(from_bits(nb));
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-3.0, 3.0);
  for (int i = 0; i < 400000; ++i) v.push_back(from_bits(rng()));
  for (int i = 0; i < 400000; ++i) v.push_back(u(rng));

  for (double a : v) {
    expect(above1(a), a > 1.0, "above1", a);
    expect(below0(a), a < 0.0, "below0", a);
    expect(above0(a), a > 0.0, "above0", a);
    expect(is0(a), a == 0.0, "is0", a);
    expect(is1(a), a == 1.0, "is1", a);
    expect(nonneg(a), a >= 0.0, "nonneg", a);
    expect(abs_above_half(a), std::fabs(a) > 0.5, "abs_above_half", a);
    expect(out01(a), a > 1.0 || a < 0.0, "out01", a);
    expect(isnan_bits(a), std::isnan(a), "isnan_bits", a);
  }
  // pairs: random, equal, opposite signs, both zeros, NaN
  const size_t n = v.size();
  for (size_t i = 0; i < n; ++i) {
    const double a = v[i];
    for (double b : {v[(i * 7919 + 13) % n], v[(i * 104729 + 1) % n], a, -a, 0.0, -0.0, qnan}) {
      expect(lt_any(a, b), a < b, "lt_any", a, b);
      expect(eq_any(a, b), a == b, "eq_any", a, b);
      if (a > 0.0 && b > 0.0) expect(pos_lt(a, b), a < b, "pos_lt", a, b);
    }
  }
  // the end of the interval: maxTime >= +0 (range test) and the others (compare)
  for (double m : {0.0, -0.0, 1.0, 130.0, 129.99999999999997, 1e300, inf, -1.0, -inf, qnan,
                   std::numeric_limits<double>::denorm_min()})
    for (double t : v) expect(past_end(m, t), m < t, "past_end", m, t);
  // the Irwin-Hall normal: every boundary of the 36-bit sum and random sums
  std::vector<unsigned long long> sums = {0ULL, 1ULL, (6ULL << 32) - 1, 6ULL << 32, (6ULL << 32) + 1,
                                          12ULL * 0xFFFFFFFFULL, 1ULL << 32, (1ULL << 35) - 1, 1ULL << 35};
  for (int e = 0; e < 36; ++e)
    for (long long d : {-1LL, 0LL, 1LL}) {
      const long long s1 = (6LL << 32) + (1LL << e) + d, s2 = (6LL << 32) - (1LL << e) + d;
      if (s1 >= 0 && s1 <= 12LL * 0xFFFFFFFFLL) sums.push_back((unsigned long long)s1);
      if (s2 >= 0 && s2 <= 12LL * 0xFFFFFFFFLL) sums.push_back((unsigned long long)s2);
    }
  std::uniform_int_distribution<unsigned long long> us(0ULL, 12ULL * 0xFFFFFFFFULL);
  for (int i = 0; i < 1000000; ++i) sums.push_back(us(rng));
  for (unsigned long long s : sums) {
    const double ref = from_bits(0x4130000000000000ULL | s) - 1048582.0;  // 2^20 + s*2^-32 - (2^20 + 6)
    const double got = ih12_normal(s);
    ++g_checked;
    if (bits(got) != bits(ref) && g_bad++ < 20)
      std::printf("MISMATCH ih12_normal sum=%llu got %a want %a\n", s, got, ref);
  }
  if (g_bad) {
    std::printf("%lld mismatches of %lld\n", g_bad, g_checked);
    return 1;
  }
  std::printf("ok %lld\n", g_checked);
  return 0;
}
