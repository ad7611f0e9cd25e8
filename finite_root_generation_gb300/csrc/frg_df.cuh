// Double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits, computed entirely
// on the FP32 pipes. GB300's FP64 rate is 1/64 of its FP32 rate, so the FP32 stage
// keeps its points and refinement residuals in df instead of FP64.
//
// Built from the error-free transformations two-sum (Knuth, TAOCP vol. 2, 4.2.2) and
// two-product via a fused multiply-add (the FMA form of Dekker's product, T. J.
// Dekker, "A floating-point technique for extending the available precision",
// Numer. Math. 18, 1971). Addition is Dekker's add2 (one two-sum of the leading parts,
// the trailing parts added in, one renormalisation): its error is at most about
// u^2 (|x| + |y|) with u = 2^-24, i.e. it perturbs each operand by a relative u^2, which is
// the backward-error form the residuals and eliminations here rely on. The complex
// operations evaluate a*b -/+ c*d with one two-sum of the two leading products and the
// cross terms folded into the trailing part (error about u^2 (|a b| + |c d|)).
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
  float s, e;
  df_two_sum(x.hi, y.hi, s, e);
  e += x.lo + y.lo;
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

// ---------------------------------------------------------------- complex double-float
#include "frg_complex.cuh"

// a*b + sgn*c*d (sgn = +1 or -1), one renormalisation
__device__ __forceinline__ df df_dot2(df a, df b, df c, df d, float sgn) {
  const float p1 = a.hi * b.hi, e1 = fmaf(a.hi, b.hi, -p1);
  const float cs = sgn * c.hi, cl = sgn * c.lo;
  const float p2 = cs * d.hi, e2 = fmaf(cs, d.hi, -p2);
  float s, t;
  df_two_sum(p1, p2, s, t);
  t += e1 + e2;
  t = fmaf(a.hi, b.lo, t);
  t = fmaf(a.lo, b.hi, t);
  t = fmaf(cs, d.lo, t);
  t = fmaf(cl, d.hi, t);
  df_quick_two_sum(s, t, s, t);
  return df(s, t);
}
// z + a*b + sgn*c*d
__device__ __forceinline__ df df_dot2_acc(df z, df a, df b, df c, df d, float sgn) {
  const float p1 = a.hi * b.hi, e1 = fmaf(a.hi, b.hi, -p1);
  const float cs = sgn * c.hi, cl = sgn * c.lo;
  const float p2 = cs * d.hi, e2 = fmaf(cs, d.hi, -p2);
  float s, t, s2, t2;
  df_two_sum(p1, p2, s, t);
  df_two_sum(s, z.hi, s2, t2);
  t += t2 + z.lo + e1 + e2;
  t = fmaf(a.hi, b.lo, t);
  t = fmaf(a.lo, b.hi, t);
  t = fmaf(cs, d.lo, t);
  t = fmaf(cl, d.hi, t);
  df_quick_two_sum(s2, t, s2, t);
  return df(s2, t);
}
// 1 / y: an approximate FP32 reciprocal with one correction from the exact residual
__device__ __forceinline__ df df_rcp(df y) {
  const float q1 = 1.0f / y.hi;
  const float p = y.hi * q1, e = fmaf(y.hi, q1, -p);
  const float r = ((1.0f - p) - e) - y.lo * q1;  // 1 - p is exact (Sterbenz)
  const float q2 = r * q1;
  float s, t;
  df_quick_two_sum(q1, q2, s, t);
  return df(s, t);
}

// The complex operations are real calls, not inlined: the refinement residual is a
// straight-line sequence of ~120 of them, and inlining every one makes its code about
// 77 KB, which evicts the FP32 step from the instruction cache; as calls it is ~30 KB.
static __device__ __noinline__ cx<df> df_cadd(cx<df> a, cx<df> b) { return cx<df>(a.re + b.re, a.im + b.im); }
static __device__ __noinline__ cx<df> df_csub(cx<df> a, cx<df> b) { return cx<df>(a.re - b.re, a.im - b.im); }
static __device__ __noinline__ cx<df> df_cmul(cx<df> a, cx<df> b) {
  return cx<df>(df_dot2(a.re, b.re, a.im, b.im, -1.f), df_dot2(a.re, b.im, a.im, b.re, 1.f));
}
__device__ __forceinline__ cx<df> operator+(cx<df> a, cx<df> b) { return df_cadd(a, b); }
__device__ __forceinline__ cx<df> operator-(cx<df> a, cx<df> b) { return df_csub(a, b); }
__device__ __forceinline__ cx<df> operator*(cx<df> a, cx<df> b) { return df_cmul(a, b); }
__device__ __forceinline__ cx<df> operator*(df s, cx<df> a) { return cx<df>(s * a.re, s * a.im); }
__device__ __forceinline__ cx<df> operator*(cx<df> a, df s) { return cx<df>(s * a.re, s * a.im); }
__device__ __forceinline__ cx<df>& operator+=(cx<df>& a, cx<df> b) { a = a + b; return a; }
__device__ __forceinline__ cx<df>& operator-=(cx<df>& a, cx<df> b) { a = a - b; return a; }
// a - b*c
static __device__ __noinline__ cx<df> cfms(cx<df> a, cx<df> b, cx<df> c) {
  return cx<df>(df_dot2_acc(a.re, -b.re, c.re, b.im, c.im, 1.f), df_dot2_acc(a.im, -b.re, c.im, b.im, c.re, -1.f));
}
// a + b*c
static __device__ __noinline__ cx<df> cfma(cx<df> b, cx<df> c, cx<df> a) {
  return cx<df>(df_dot2_acc(a.re, b.re, c.re, b.im, c.im, -1.f), df_dot2_acc(a.im, b.re, c.im, b.im, c.re, 1.f));
}
__device__ __forceinline__ df cnorm2(cx<df> a) { return df_dot2(a.re, a.re, a.im, a.im, 1.f); }
// 1/b = conj(b) / |b|^2 (the tracker's operands are far from the FP32 range limits)
static __device__ __noinline__ cx<df> cinv(cx<df> b) {
  const df r = df_rcp(cnorm2(b));
  return cx<df>(b.re * r, -(b.im * r));
}
__device__ __forceinline__ cx<df> cdiv(cx<df> a, cx<df> b) { return a * cinv(b); }

