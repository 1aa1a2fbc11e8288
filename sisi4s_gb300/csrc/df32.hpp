// Float-float ("double-single") arithmetic: a value is hi + lo with two FP32
// numbers, |lo| <= ulp(hi)/2, about 48 significant bits.  Used where FP64
// accuracy is needed for elementwise work: on this GPU the FP32 pipe issues
// ~64x as many operations per clock as the FP64 pipe, and one float-float
// operation costs 3-15 FP32 instructions.
//
// The sums use Knuth's TwoSum and Dekker's Fast2Sum; the products use the
// FMA-based exact product (Dekker / Ogita-Rump-Oishi).  The add is the
// "sloppy" variant (error <= ~2^-46 of the larger operand, not of the
// result); the division is Newton-style long division with three FP32
// quotient digits.  Built without fast-math, so the compiler keeps every
// rounding these error-free transformations rely on.
#pragma once

#include <cuda_runtime.h>

namespace gbcc {

struct __align__(8) df32 {
  float hi, lo;
};

__host__ __device__ __forceinline__ df32 df_make(float hi, float lo) {
  df32 r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// (s, e) with |e| <= ulp(s)/2 -> normalized pair (requires |s| >= |e|)
__device__ __forceinline__ df32 df_fast2sum(float s, float e) {
  const float h = s + e;
  return df_make(h, e - (h - s));
}

__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
  return df_fast2sum(s, e);
}

__device__ __forceinline__ df32 df_neg(df32 a) { return df_make(-a.hi, -a.lo); }

__device__ __forceinline__ df32 df_sub(df32 a, df32 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast2sum(p, e);
}

// a * b for an FP32 b
__device__ __forceinline__ df32 df_mulf(df32 a, float b) {
  const float p = a.hi * b;
  const float e = fmaf(a.lo, b, fmaf(a.hi, b, -p));
  return df_fast2sum(p, e);
}

// a / b: three FP32 quotient digits, each from the exact-enough remainder
__device__ __forceinline__ df32 df_div(df32 a, df32 b) {
  const float q1 = __fdividef(a.hi, b.hi);
  const df32 r1 = df_sub(a, df_mulf(b, q1));
  const float q2 = __fdividef(r1.hi, b.hi);
  const df32 r2 = df_sub(r1, df_mulf(b, q2));
  const float q3 = __fdividef(r2.hi, b.hi);
  return df_add(df_fast2sum(q1, q2), df_make(q3, 0.0f));
}

__host__ __device__ __forceinline__ double df_to_double(df32 a) {
  return (double)a.hi + (double)a.lo;
}

// nearest pair to a double (FP64 instructions: for set-up work, not loops)
__host__ __device__ __forceinline__ df32 df_from_double(double x) {
  const float h = (float)x;
  return df_make(h, (float)(x - (double)h));
}

}  // namespace gbcc
