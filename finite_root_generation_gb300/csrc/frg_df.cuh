// Double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits, computed entirely
// on the FP32 pipes. GB300's FP64 rate is 1/64 of its FP32 rate, so the FP32 stage
// keeps its points and refinement residuals in df instead of FP64.
//
// Built from the error-free transformations two-sum (Knuth, TAOCP vol. 2, 4.2.2) and
// two-product via a fused multiply-add (the FMA form of Dekker's product, T. J.
// Dekker, "A floating-point technique for extending the available precision",
// Numer. Math. 18, 1971); addition renormalises both components (the accurate,
// cancellation-safe variant), division takes two quotient corrections.
#pragma once

#include <cuda_runtime.h>

struct df {
  float hi, lo;
  __host__ __device__ __forceinline__ df() {}
  __host__ __device__ __forceinline__ constexpr df(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ __forceinline__ constexpr df(float x) : hi(x), lo(0.f) {}
  __host__ __device__ __forceinline__ constexpr df(int x) : hi(float(x)), lo(0.f) {}
  // from double: the leading float and the rounded remainder (exact for the constants
  // the compiler folds; at run time it costs two FP64 operations)
  __host__ __device__ __forceinline__ constexpr df(double d) : hi(float(d)), lo(float(d - double(float(d)))) {}
  __host__ __device__ __forceinline__ explicit operator float() const { return hi + lo; }
  __host__ __device__ __forceinline__ explicit operator double() const { return double(hi) + double(lo); }
};

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void df_quick_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

__device__ __forceinline__ df operator+(df x, df y) {
  float s, e, t, f;
  df_two_sum(x.hi, y.hi, s, e);
  df_two_sum(x.lo, y.lo, t, f);
  e += t;
  df_quick_two_sum(s, e, s, e);
  e += f;
  df_quick_two_sum(s, e, s, e);
  return df(s, e);
}
__device__ __forceinline__ df operator-(df x) { return df(-x.hi, -x.lo); }
__device__ __forceinline__ df operator-(df x, df y) { return x + (-y); }
__device__ __forceinline__ df operator*(df x, df y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  float s, r;
  df_quick_two_sum(p, e, s, r);
  return df(s, r);
}
__device__ __forceinline__ df operator/(df x, df y) {
  const float q1 = x.hi / y.hi;
  df r = x - y * df(q1);
  const float q2 = r.hi / y.hi;
  r = r - y * df(q2);
  const float q3 = r.hi / y.hi;
  float s, e;
  df_quick_two_sum(q1, q2, s, e);
  return df(s, e) + df(q3);
}
__device__ __forceinline__ df& operator+=(df& x, df y) { x = x + y; return x; }
__device__ __forceinline__ df& operator-=(df& x, df y) { x = x - y; return x; }
__device__ __forceinline__ df fma(df a, df b, df c) { return a * b + c; }
__device__ __forceinline__ bool operator<(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df a, df b) { return b < a; }
__device__ __forceinline__ bool operator>=(df a, df b) { return !(a < b); }
__device__ __forceinline__ bool operator<=(df a, df b) { return !(b < a); }
__device__ __forceinline__ df sqrt(df a) {
  // one Newton step on the float square root
  const float r = sqrtf(a.hi);
  if (r == 0.f) return df(0.f);
  const df rr = df(r);
  return rr + (a - rr * rr) / df(2.f * r);
}
__device__ __forceinline__ df fmax(df a, df b) { return a < b ? b : a; }
__device__ __forceinline__ df fmin(df a, df b) { return a < b ? a : b; }
