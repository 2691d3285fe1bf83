// te_df64.cuh -- float-float ("double-FP32") arithmetic for the outer Krylov
// loop of the mixed-precision solve.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so FP64 stencils, vector updates
// and dot products are FP64-pipe bound, not HBM bound.  A value here is an
// unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, about
// 48 significant bits (relative precision ~1.4e-14) -- enough for a 1e-10
// relative residual -- computed on the FP32 pipes.
//
// The algorithms are the published error-free transformations:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971),
//   TwoProd via fused multiply-add, and the double-double addition and
//   multiplication built from them (Dekker 1971; Hida, Li and Bailey,
//   "Algorithms for quad-double precision floating point arithmetic", 2001).
// They need IEEE round-to-nearest FP32 without reassociation (the default
// nvcc flags; fused multiply-adds only ever make the products more exact).
//
// Vectors are stored as two FP32 arrays, hi and lo, so the hi half of a
// Krylov vector is a plain FP32 level buffer the FP32 V-cycle reads directly.
#pragma once
#include <cuda_runtime.h>

namespace te {

struct df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  // nearest split of a double (also usable in constant expressions, e.g. 1/3)
  __host__ __device__ constexpr df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__host__ __device__ __forceinline__ df64 df_from_double(double d) { return df64(d); }

// The split df64(d) -- hi = RN(d), lo = RN(d - hi) in FP32 -- by integer
// operations, for the bulk conversions of FP64 vectors: on GB300 every
// FP64<->FP32 conversion runs on the FP64 pipe.  With d = (-1)^s M 2^(E-52),
// M the 53-bit significand: hi keeps M's top 24 bits rounded to nearest even
// (a carry moves it to the next binade), the remainder d - hi is the integer
// r = (M mod 2^29) - [rounded up] 2^29 times 2^(E-52), and RN(r) as an FP32
// integer conversion scaled by the exact power 2^(E-52) is RN(d - hi).  Used
// when E is in [-74, 126], so hi and a nonzero lo are normal FP32 numbers;
// zeros are (+-0, +0) as in the formula; other values (subnormals, huge, Inf,
// NaN) take the FP64 formula.
__host__ __device__ __forceinline__ df64 df_split_bits(double d) {
  unsigned long long b;
#ifdef __CUDA_ARCH__
  b = (unsigned long long)__double_as_longlong(d);
#else
  __builtin_memcpy(&b, &d, 8);
#endif
  // zeros (the ghost cells of a padded level are): (+-0, +0), as the formula gives, without it
  if ((b << 1) == 0) return df64((b >> 63) ? -0.f : 0.f, 0.f);
  const int E = (int)((b >> 52) & 0x7ff) - 1023;
  if (E < -74 || E > 126) return df64(d);
  const unsigned long long M = (b & ((1ull << 52) - 1)) | (1ull << 52);
  const unsigned long long rem = M & ((1ull << 29) - 1);
  unsigned long long q = M >> 29;  // 24 bits
  const unsigned long long half = 1ull << 28;
  const int up = (rem > half || (rem == half && (q & 1))) ? 1 : 0;
  q += up;
  int eh = E;
  if (q == (1ull << 24)) {
    q >>= 1;
    eh += 1;
  }
  const unsigned int sign = (unsigned int)(b >> 63) << 31;
  const unsigned int hb = sign | ((unsigned int)(eh + 127) << 23) | (unsigned int)(q & 0x7fffff);
  // the remainder with d's sign (an exact zero stays +0, as RN(d - hi) gives)
  const long long r0 = (long long)rem - (up ? (1ll << 29) : 0ll);
  const int r = (int)(sign ? -r0 : r0);
  const unsigned int pb = (unsigned int)(E - 52 + 127) << 23;  // 2^(E-52), a normal FP32 power of two
  float hi, lo, pw;
#ifdef __CUDA_ARCH__
  hi = __uint_as_float(hb);
  pw = __uint_as_float(pb);
  lo = __int2float_rn(r) * pw;
#else
  __builtin_memcpy(&hi, &hb, 4);
  __builtin_memcpy(&pw, &pb, 4);
  lo = (float)r * pw;
#endif
  return df64(hi, lo);
}
__host__ __device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

// (double)f built from f's bits with integer operations (the exponent rebiased from 127 to
// 1023, the significand shifted into place), exact like the conversion; zeros keep their sign.
// Subnormal, infinite and NaN values take the conversion instruction.  On GB300 the conversion
// runs on the FP64 pipe (1/64 of the FP32 rate); this form does not.
__host__ __device__ __forceinline__ double f2d_bits(float f) {
  unsigned int u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  __builtin_memcpy(&u, &f, 4);
#endif
  const unsigned int e = (u >> 23) & 0xff, m = u & 0x7fffff;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  unsigned long long b;
  if (e == 0 && m == 0) {
    b = sign;
  } else if (e == 0 || e == 255) {
    return (double)f;
  } else {
    b = sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)m << 29);
  }
  double d;
#ifdef __CUDA_ARCH__
  d = __longlong_as_double((long long)b);
#else
  __builtin_memcpy(&d, &b, 8);
#endif
  return d;
}
// df_to_double with the conversions done by f2d_bits: the same value, one FP64 addition
__host__ __device__ __forceinline__ double df_to_double_bits(df64 a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

// s + e == a + b exactly
__device__ __forceinline__ df64 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df64{s, e};
}
// s + e == a + b exactly when |a| >= |b|
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df64{s, e};
}
// p + e == a * b exactly
__device__ __forceinline__ df64 two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return df64{p, e};
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  df64 t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64{-a.hi, -a.lo}; }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
// df64 * FP32 value
__device__ __forceinline__ df64 operator*(df64 a, float b) {
  df64 p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
// a * x + b * y for FP32 x, y: both products' high parts summed exactly
// (TwoProd, TwoSum), every low-order term collected in one FP32 sum, then
// renormalised.  The error is about 2^-47 (|a x| + |b y|), the same order as
// forming the two products and their float-float sum separately, at less
// than half the operations.
__device__ __forceinline__ df64 df_sum2(df64 a, float x, df64 b, float y) {
  const df64 p = two_prod(a.hi, x), q = two_prod(b.hi, y);
  const df64 t = two_sum(p.hi, q.hi);
  float lo = __fadd_rn(t.lo, __fadd_rn(p.lo, q.lo));
  lo = __fmaf_rn(a.lo, x, lo);
  lo = __fmaf_rn(b.lo, y, lo);
  return fast_two_sum(t.hi, lo);
}
// a * x + b * y for float-float x, y (the cross terms a.hi x.lo + a.lo x.hi
// of each product join the low-order sum)
__device__ __forceinline__ df64 df_sum2(df64 a, df64 x, df64 b, df64 y) {
  const df64 p = two_prod(a.hi, x.hi), q = two_prod(b.hi, y.hi);
  const df64 t = two_sum(p.hi, q.hi);
  float lo = __fadd_rn(t.lo, __fadd_rn(p.lo, q.lo));
  lo = __fmaf_rn(a.hi, x.lo, lo);
  lo = __fmaf_rn(a.lo, x.hi, lo);
  lo = __fmaf_rn(b.hi, y.lo, lo);
  lo = __fmaf_rn(b.lo, y.hi, lo);
  return fast_two_sum(t.hi, lo);
}

// Dot-product accumulator after Ogita, Rump and Oishi, "Accurate sum and dot
// product" (SIAM J. Sci. Comput. 26(6), 2005), algorithm Dot2, with
// float-float factors: the running FP32 sum s takes each product's high part
// through TwoSum, and c collects the rounding errors of those additions, the
// products' low parts (TwoProd) and the cross terms.  The value s + c is kept
// as a float-float number (not rounded to FP32), so for n terms its error is
// about n^2 2^-48 sum |a_i b_i|: far below what the 1e-10 stopping test
// resolves, at half the operations of a float-float multiply and add per term.
struct dot2 {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(df64 a, df64 b) {
    const df64 p = two_prod(a.hi, b.hi);
    const float cross = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
    const df64 t = two_sum(s, p.hi);
    s = t.hi;
    c = __fadd_rn(c, __fadd_rn(t.lo, __fadd_rn(p.lo, cross)));
  }
  __device__ __forceinline__ df64 value() const { return two_sum(s, c); }
};

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }

__device__ __forceinline__ df64 df_shfl_down(df64 v, int o) {
  return df64{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

}  // namespace te
