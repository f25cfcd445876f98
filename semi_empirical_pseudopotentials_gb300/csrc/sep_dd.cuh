// sep_dd.cuh -- double-float arithmetic: a value is the unevaluated sum of two
// floats hi + lo (|lo| <= ulp(hi) / 2), about 48 significant bits, on the
// FP32 pipe.  On GB300 the FP32 pipe issues 64 times the FP64 pipe's rate, so
// FFT passes whose FP64 form is bound by the FP64 pipe run several times
// faster in this form at close to FP64 accuracy (relative rounding about
// 2^-47 per operation against FP64's 2^-53).
//
// The operations are the error-free transformations of Knuth (TwoSum) and
// Dekker (FastTwoSum), with TwoProd by a fused multiply-add, combined as in
// the double-double literature (Hida, Li and Bailey, "Algorithms for quad-
// double precision floating point arithmetic", 2001): "sloppy" addition
// (error bounded relative to |a| + |b|, enough for the normwise error of an
// FFT) and multiplication with the cross terms folded into the product's
// error.  Every step uses the round-to-nearest intrinsics, so the compiler
// neither contracts nor reorders them.
#pragma once

#include "sep_dft.cuh"

namespace sep {

struct ddf {
  float hi, lo;
  ddf() = default;
  __host__ __device__ constexpr ddf(float h, float l) : hi(h), lo(l) {}
  // nearest split of a double: hi = fl(d), lo = fl(d - hi)
  __host__ __device__ constexpr ddf(double d)
      : hi(static_cast<float>(d)), lo(static_cast<float>(d - static_cast<double>(static_cast<float>(d)))) {}
  __host__ __device__ constexpr double to_double() const {
    return static_cast<double>(hi) + static_cast<double>(lo);
  }
  __host__ __device__ constexpr explicit operator double() const { return to_double(); }
};

struct __align__(16) cddf {
  ddf x, y;
};
template <> struct cvec<ddf> { using type = cddf; };

namespace dd {
// s + e = a + b exactly
__device__ __forceinline__ ddf two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ddf(s, e);
}
// s + e = a + b exactly when |a| >= |b| (or a = 0)
__device__ __forceinline__ ddf fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return ddf(s, __fsub_rn(b, __fsub_rn(s, a)));
}
}  // namespace dd

__device__ __forceinline__ ddf operator+(ddf a, ddf b) {
  const ddf s = dd::two_sum(a.hi, b.hi);
  return dd::fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ddf operator-(ddf a) { return ddf(-a.hi, -a.lo); }
__device__ __forceinline__ ddf operator-(ddf a, ddf b) { return a + (-b); }
__device__ __forceinline__ ddf operator*(ddf a, ddf b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // the product's rounding error
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dd::fast_two_sum(p, e);
}
__device__ __forceinline__ ddf& operator+=(ddf& a, ddf b) { return a = a + b; }
__device__ __forceinline__ ddf& operator-=(ddf& a, ddf b) { return a = a - b; }
__device__ __forceinline__ bool operator>(ddf a, ddf b) {
  return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}
__device__ __forceinline__ ddf fma_t(ddf a, ddf b, ddf c) { return a * b + c; }

}  // namespace sep
