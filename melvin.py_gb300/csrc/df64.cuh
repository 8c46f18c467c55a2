// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)/2), giving a 48-bit significand.
//
// The operations are the classic error-free transformations (Knuth's
// two-sum, Dekker/Kahan's fast two-sum, FMA-based exact products) as
// published by Dekker (1971), Knuth (TAOCP vol. 2) and Hida, Li & Bailey
// (2001).  Every step uses explicitly rounded intrinsics so the compiler
// neither contracts nor reassociates them.
//
// Accuracy: addition is the "sloppy" variant, with absolute error about
// 2^-47 (|a| + |b|); multiplication has relative error about 2^-46.  That is
// the error model of an FFT (errors relative to the input norm), so an FFT
// computed in df64 is accurate to ~1e-14 relative L2 while running on the
// FP32 pipes, which issue about 60x faster than FP64 on GB300.
//
// Addition and multiplication leave their results unnormalised: the sum
// keeps the exact two-sum of the high words and adds the low words into its
// error term (8 FP32 operations instead of 11), the product keeps the exact
// product of the high words and accumulates the cross terms into its error
// term (4 instead of 7), without the final fast two-sum.  The low word may
// then grow by a few ulps of the high one per operation; two-sum and the
// FMA products are exact for any operands, the transforms renormalise every
// value once per pass (pass_out in fft_block.cuh), so the pair keeps ~46
// bits, and the conversion to double adds the halves exactly.
//
// The exponent range is FP32's: magnitudes below ~1e-30 lose low bits and
// values below 1e-38 flush, which is far outside the range of the fields
// transformed here.
#pragma once

#include <cuda_runtime.h>

namespace mgb {

struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  // Construction from a double (constant-folded for literals).
  __host__ __device__ constexpr df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df64(s, e);
}

// Renormalise (hi, lo) to |lo| <= ulp(hi)/2: Dekker's fast two-sum, exact
// when hi's exponent is at least lo's (the usual case: lo holds a few ulps
// of hi); after a cancellation that left lo the larger, the error is
// relative to that small value.
__device__ __forceinline__ df64 df_renorm(df64 a) {
  const float s = __fadd_rn(a.hi, a.lo);
  return df64(s, __fsub_rn(a.lo, __fsub_rn(s, a.hi)));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = df_two_sum(a.hi, b.hi);
  return df64(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }

__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df64(p, e);
}

}  // namespace mgb
