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
__host__ __device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

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
