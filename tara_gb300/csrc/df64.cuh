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
// Unnormalised forms for chains inside one butterfly: the value is still hi + lo
// exactly, but lo is not folded into hi's last place, which saves the
// FastTwoSum (3 of the 11 operations of an add, 3 of the 7 of a multiply).
// mul_u takes normalised operands (values read from shared memory, twiddles);
// every chain ends in renorm() before its result is stored.  The error stays
// bounded relative to the operands' magnitudes, as for the sloppy add.
__device__ __forceinline__ df64 add_u(df64 a, df64 b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return df64(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df64 sub_u(df64 a, df64 b) { return add_u(a, -b); }
__device__ __forceinline__ df64 mul_u(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df64(p, e);
}
__device__ __forceinline__ df64 renorm(df64 a) {
  df64 r;
  fast_two_sum(a.hi, a.lo, r.hi, r.lo);
  return r;
}

struct __align__(16) df64c {
  df64 x, y;
};

// Conversions between double and df64 by integer operations on the bit
// patterns: on GB300 every FP64-pipe instruction (including F2F conversions)
// issues at 2 per SM per cycle, so the kernels that read the FP64 state split
// it without touching that pipe.
//
// double -> df64: hi = the double truncated to 24 significant bits (exact),
// lo = the remaining 29 bits rounded to 24, so hi + lo = d within 2^-48 |d|.
// Magnitudes below 2^-126 become 0 (absolute error < 2^-126); lo is dropped
// below 2^-74 (absolute error < 2^-98); infinities and NaNs map to FP32 ones.
__device__ __forceinline__ df64 split_double(double d) {
  const unsigned int hw = (unsigned int)__double2hiint(d), lw = (unsigned int)__double2loint(d);
  const unsigned int sgn = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7ffu);  // biased double exponent
  const unsigned int top = ((hw & 0xfffffu) << 3) | (lw >> 29);  // 23 mantissa bits after the leading 1
  if (e > 1150) {  // beyond the FP32 range: infinity, or NaN (mantissa kept non-zero)
    const unsigned int nan = (e == 2047 && ((hw & 0xfffffu) | lw)) ? 0x400000u : 0u;
    return df64(__uint_as_float(sgn | 0x7f800000u | nan), 0.f);
  }
  if (e < 897) return df64(__uint_as_float(sgn), 0.f);
  const float hi = __uint_as_float(sgn | ((unsigned int)(e - 896) << 23) | top);
  float lo = 0.f;
  if (e >= 949) {
    const unsigned int m = lw & 0x1fffffffu;  // 29 bits below hi's last bit
    // exact FP32 values of the two parts of m (each below 2^23) by the 2^23 bias trick
    const float mh = __fsub_rn(__uint_as_float(0x4b000000u | (m >> 23)), 8388608.f);
    const float ml = __fsub_rn(__uint_as_float(0x4b000000u | (m & 0x7fffffu)), 8388608.f);
    const float fm = __fmaf_rn(mh, 8388608.f, ml);                        // m, rounded to 24 bits
    const float scale = __uint_as_float((unsigned int)(e - 948) << 23);  // 2^(e - 1075)
    lo = __uint_as_float(__float_as_uint(__fmul_rn(fm, scale)) | sgn);
  }
  return df64(hi, lo);
}

// FP32 value -> the bits of the equal double (exact), by integer operations.
__device__ __forceinline__ double float_bits_to_double(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int sgn = b & 0x80000000u, ef = (b >> 23) & 0xffu, mf = b & 0x7fffffu;
  if (ef == 0u) return __hiloint2double((int)sgn, 0);  // zero (subnormals flush to 0)
  const unsigned int ed = ef == 0xffu ? 0x7ffu : ef + 896u;
  return __hiloint2double((int)(sgn | (ed << 20) | (mf >> 3)), (int)(mf << 29));
}

// df64 -> double: both parts widened exactly, one FP64 add.
__device__ __forceinline__ double to_double(df64 a) {
  return float_bits_to_double(a.hi) + float_bits_to_double(a.lo);
}

}  // namespace tara
