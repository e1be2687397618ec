// df.cuh -- float-float ("double-single") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, giving about 48
// significant bits.  The error-free transformations are the published ones: TwoSum (Knuth, TAOCP
// vol. 2, 4.2.2), Fast-TwoSum (Dekker 1971) and TwoProduct via a fused multiply-add; addition is the
// "sloppy" double-single sum of Dekker / the QD library (Hida, Li, Bailey 2001), whose error is
// bounded by a few units of 2^-48 relative to the sum of the operand magnitudes.
// GB300's FP64 pipe runs at 1/58 of its FP32 rate; an element kernel in this arithmetic computes
// FP64-accurate element matrices on the FP32 pipes.
#pragma once

#include <cuda_runtime.h>

struct f2 {
  float hi, lo;
};

__device__ __forceinline__ f2 f2_from(double a) {
  const float h = (float)a;
  return {h, (float)(a - (double)h)};
}
__device__ __forceinline__ f2 f2_from(float a) { return {a, 0.0f}; }
__device__ __forceinline__ double f2_to_double(f2 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ f2 fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  f2 s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}

__device__ __forceinline__ f2 operator-(f2 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return a + (-b); }

// Product without the final renormalisation: |lo| stays within a few units of ulp(hi), which the
// sum and product formulas tolerate (they never rely on |lo| <= ulp(hi)/2).
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return {p, e};
}

// Accumulation without renormalising after every term: the high parts are summed exactly with
// TwoSum and the (small) rounding errors and low parts are gathered in `lo`; finish() restores the
// normal form.  Used for sums of a modest number of terms.
__device__ __forceinline__ void accum(f2& acc, f2 t) {
  const f2 s = two_sum(acc.hi, t.hi);
  acc.hi = s.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ void accum_sub(f2& acc, f2 t) { accum(acc, f2{-t.hi, -t.lo}); }
__device__ __forceinline__ void finish(f2& acc) { acc = two_sum(acc.hi, acc.lo); }
__device__ __forceinline__ void accum(double& acc, double t) { acc += t; }
__device__ __forceinline__ void accum_sub(double& acc, double t) { acc -= t; }
__device__ __forceinline__ void finish(double&) {}
__device__ __forceinline__ void accum(float& acc, float t) { acc += t; }
__device__ __forceinline__ void accum_sub(float& acc, float t) { acc -= t; }
__device__ __forceinline__ void finish(float&) {}

__device__ __forceinline__ f2& operator+=(f2& a, f2 b) { return a = a + b; }
__device__ __forceinline__ f2& operator-=(f2& a, f2 b) { return a = a - b; }
__device__ __forceinline__ bool operator>(f2 a, f2 b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

// 1/sqrt(x): FP32 estimate refined by one Newton step y <- y + y (1 - x y^2) / 2 in float-float
// (quadratic convergence from ~2^-23 to ~2^-46).
__device__ __forceinline__ f2 rsqrt(f2 x) {
  const float y0 = rsqrtf(x.hi);
  const f2 y = {y0, 0.0f};
  const f2 r = f2{1.0f, 0.0f} - x * (y * y);
  return y + y * (r * f2{0.5f, 0.0f});
}

// Exact float -> double conversion by re-packing the IEEE-754 fields with integer operations
// (sign, exponent rebiased by 1023 - 127 = 896, mantissa shifted into the top of the 52-bit
// field).  GB300 executes floating-point conversions on its narrow FP64 pipe; this form keeps the
// FP32-pipe kernels off it.  Zeros are handled here, subnormals, infinities and NaNs fall back to
// the hardware conversion.
__device__ __forceinline__ double f32_to_f64_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
  if (e == 0u) {
    if ((u & 0x7fffffu) == 0u) return __longlong_as_double((long long)sgn);
    return (double)f;
  }
  if (e == 0xffu) return (double)f;
  const unsigned long long bits =
      sgn | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// precision-generic helpers used by the element kernels
template <typename T>
__device__ __forceinline__ T from_double(double a) {
  return (T)a;
}
template <>
__device__ __forceinline__ f2 from_double<f2>(double a) {
  return f2_from(a);
}
__device__ __forceinline__ double to_double(double a) { return a; }
__device__ __forceinline__ double to_double(float a) { return (double)a; }
__device__ __forceinline__ double to_double(f2 a) { return f2_to_double(a); }
