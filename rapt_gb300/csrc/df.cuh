// df.cuh -- float-float ("double-float") arithmetic on the FP32 pipe.
//
// A value is an unevaluated sum hi + lo of two floats (~48-bit significand).
// Error-free transformations: TwoSum (Knuth), FastTwoSum (Dekker, |a| >= |b|),
// and the FMA-based TwoProd (Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26, 2005).
// Reciprocal and reciprocal square root: one Newton-Raphson step from the FP32
// approximation, with the residual formed in float-float.
// On GB300 one FP32 FMA issues at 64x the FP64 rate, so a float-float
// operation (4-20 FP32 instructions) costs a fraction of one FP64 operation.
#pragma once
#include <cuda_runtime.h>

namespace rapt {

struct DF {
  float hi, lo;
};

__device__ __forceinline__ DF df(float a) { return DF{a, 0.f}; }
__device__ __forceinline__ DF df_from_double(double v) {
  const float h = (float)v;
  return DF{h, (float)(v - (double)h)};
}
__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ float df_f(DF a) { return a.hi + a.lo; }

__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return DF{s, __fadd_rn(b, -__fadd_rn(s, -a))};
}
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  return DF{s, __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb))};
}
__device__ __forceinline__ DF two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return DF{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ DF operator+(DF a, DF b) {
  DF s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ DF operator-(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator+(DF a, float b) {
  DF s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ DF operator*(DF a, DF b) {
  DF p = two_prod(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, e);
}
__device__ __forceinline__ DF operator*(DF a, float b) {
  DF p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// a * b + c
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) { return a * b + c; }
__device__ __forceinline__ DF df_fma(DF a, float b, DF c) { return a * b + c; }

// 1 / a: y0 = 1/a.hi (FP32), y = y0 + y0 (1 - a y0)
__device__ __forceinline__ DF df_rcp(DF a) {
  const float y0 = __frcp_rn(a.hi);
  const DF r = DF{1.f, 0.f} - a * y0;
  return fast_two_sum(y0, __fmul_rn(y0, df_f(r)));
}
__device__ __forceinline__ DF operator/(DF a, DF b) { return a * df_rcp(b); }

// 1 / sqrt(a): y0 = rsqrt(a.hi) (FP32), y = y0 + y0 (1 - a y0^2) / 2
__device__ __forceinline__ DF df_rsqrt(DF a) {
  const float y0 = rsqrtf(a.hi);
  const DF r = DF{1.f, 0.f} - (a * y0) * y0;
  return fast_two_sum(y0, __fmul_rn(0.5f * y0, df_f(r)));
}

__device__ __forceinline__ DF df_abs(DF a) { return (a.hi < 0.f) ? -a : a; }

}  // namespace rapt
