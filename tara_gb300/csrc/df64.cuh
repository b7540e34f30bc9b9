// Double-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits, computed on
// the FP32 pipes.  On GB300 FP64 instructions issue at 1/64 of the FP32 rate, so
// transforms written in df64 trade ~15 FP32 instructions for each FP64 one and
// still come out ahead.
//
// The error-free transformations are the classical ones: TwoSum (Knuth, TAOCP
// vol. 2, 4.2.2), FastTwoSum (Dekker 1971) and TwoProd through a fused
// multiply-add; the double-word add and multiply follow the "sloppy" forms of
// Hida, Li and Bailey, "Algorithms for quad-double precision floating point
// arithmetic" (ARITH 2001), whose error is bounded relative to the operands'
// magnitudes -- the bound an FFT's error analysis uses.  No reassociation or
// fast-math may touch these functions (the build uses neither).
#pragma once
#include <cuda_runtime.h>

namespace tara {

// The kernels call fma() unqualified for every scalar type; keep the standard
// float and double overloads visible beside the df64 one.
using ::fma;

struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ explicit df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit df64(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  df64 r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // TwoProd: the exact rounding error of p
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  df64 r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}

// a*b + c with the product's error carried into the sum
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float s, t;
  two_sum(p, c.hi, s, t);
  t = __fadd_rn(t, __fadd_rn(e, c.lo));
  df64 r;
  fast_two_sum(s, t, r.hi, r.lo);
  return r;
}

// 16-byte aligned so shared-memory and global accesses stay single vector ops
struct __align__(16) df64c {
  df64 x, y;
};

}  // namespace tara
