// Host check of df_split_bits (thunderegg_gb300/csrc/te_df64.cuh): the integer
// split of a double into float-float must equal the FP64 formula
// hi = RN(d), lo = RN(d - hi) bit for bit.  Built and run by
// tests/test_df64_split.py (host code only, no GPU).
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>

#include "te_df64.cuh"

static uint32_t fbits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

int main() {
  std::mt19937_64 g(12345);
  long long bad = 0, n = 0;
  auto check = [&](double d) {
    const te::df64 a = te::df_split_bits(d);
    const float hi = (float)d;
    const float lo = (float)(d - (double)hi);
    n++;
    if (fbits(a.hi) != fbits(hi) || fbits(a.lo) != fbits(lo)) {
      if (bad < 10) std::printf("mismatch d=%a: got (%a, %a) want (%a, %a)\n", d, a.hi, a.lo, hi, lo);
      bad++;
    }
  };
  // random bit patterns over every exponent, random values in the solver's range
  for (int i = 0; i < 2000000; i++) {
    uint64_t b = g();
    double d;
    std::memcpy(&d, &b, 8);
    if (d == d) check(d);
  }
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-80, 130);
  for (int i = 0; i < 2000000; i++) check(std::ldexp(u(g), ex(g)));
  // ties and carries: significands whose low 29 bits are exactly half, all ones or zero
  for (int i = 0; i < 200000; i++) {
    uint64_t b = g();
    const uint64_t low[4] = {1ull << 28, (1ull << 29) - 1, 0, (1ull << 28) + 1};
    b = (b & ~((1ull << 29) - 1)) | low[i & 3];
    if (i & 4) b |= ((1ull << 52) - 1) & ~((1ull << 29) - 1);  // all-ones high part: rounding carries
    double d;
    std::memcpy(&d, &b, 8);
    if (d == d) check(d);
  }
  const double special[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 1.1754943508222875e-38, 5e-324, 1e300,
                            -1e-300, 2.0e-23, 1.5, 0.1, 1.0 / 3.0};
  for (double d : special) check(d);
  std::printf("%lld of %lld splits differ\n", bad, n);
  // f2d_bits: the exact widening of every float class (normal, zero of both signs, subnormal,
  // infinite, NaN) equals the cast bit for bit
  long long badw = 0, nw = 0;
  auto checkw = [&](uint32_t fb) {
    float f;
    std::memcpy(&f, &fb, 4);
    const double a = te::f2d_bits(f), want = (double)f;
    uint64_t ab, wb;
    std::memcpy(&ab, &a, 8);
    std::memcpy(&wb, &want, 8);
    nw++;
    if (ab != wb && !(a != a && want != want)) {
      if (badw < 10) std::printf("widening mismatch f=%a: got %a want %a\n", f, a, want);
      badw++;
    }
  };
  for (uint32_t e = 0; e < 256; e++)
    for (int i = 0; i < 4000; i++) checkw((uint32_t)(g() & 0x807fffffu) | (e << 23));
  const uint32_t fspecial[] = {0u, 0x80000000u, 1u, 0x807fffffu, 0x00800000u, 0x7f7fffffu, 0x7f800000u,
                               0xff800000u, 0x7fc00000u, 0x3f800000u};
  for (uint32_t fb : fspecial) checkw(fb);
  std::printf("%lld of %lld widenings differ\n", badw, nw);
  return bad == 0 && badw == 0 ? 0 : 1;
}
