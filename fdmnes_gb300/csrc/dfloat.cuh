// dfloat.cuh - double-float arithmetic: a value is the unevaluated sum hi + lo
// of two floats (about 48 significand bits), computed on the FP32 pipes.
//
// GB300's FP64 rate is about 1/60 of its FP32 rate, so the FP64-class
// re-factorisation of an energy whose FP32 factors are too poor runs in this
// type.  Sums use Knuth's two-sum, products the exact FMA split of hi*hi plus
// the cross terms; both are renormalised (Dekker 1971, "A floating-point
// technique for extending the available precision").
#pragma once

#include <cuda_runtime.h>

namespace fdm {

struct dfl {
  float hi, lo;
  __host__ __device__ dfl() : hi(0.f), lo(0.f) {}
  __host__ __device__ dfl(float h, float l) : hi(h), lo(l) {}
  __device__ explicit dfl(double d) {
    hi = __double2float_rn(d);
    lo = __double2float_rn(d - (double)hi);
  }
  __device__ explicit dfl(int i) : hi((float)i), lo(0.f) {}
  __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return dfl(s, e);
}
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dfl(s, b - (s - a));
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  dfl s = df_two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q1 = a.hi / b.hi;
  const dfl r = a - b * dfl(q1, 0.f);
  const float q2 = r.hi / b.hi;
  return df_fast_two_sum(q1, q2);
}
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }

}  // namespace fdm
