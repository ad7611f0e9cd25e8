// Complex arithmetic for the tracker kernels, templated on the real type so the
// same code runs in FP64 (the reference's precision, classes.cuh:24-36) and FP32.
//
// Multiplication is the textbook formula with fused multiply-adds; FP32 division is
// Smith's algorithm (R. L. Smith, "Algorithm 116: Complex division", CACM 5(8),
// 1962), which avoids the overflow of the naive |b|^2 form in FP32's narrow range.
#pragma once

#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define FRG_HD __host__ __device__ __forceinline__
#else
#define FRG_HD inline
#endif

template <typename T>
struct cx {
  T re, im;
  FRG_HD cx() {}
  FRG_HD constexpr cx(T r, T i = T(0)) : re(r), im(i) {}
  template <typename U>
  FRG_HD explicit cx(const cx<U>& o) : re(T(o.re)), im(T(o.im)) {}
};

template <typename T>
FRG_HD cx<T> operator+(cx<T> a, cx<T> b) { return cx<T>(a.re + b.re, a.im + b.im); }
template <typename T>
FRG_HD cx<T> operator-(cx<T> a, cx<T> b) { return cx<T>(a.re - b.re, a.im - b.im); }
template <typename T>
FRG_HD cx<T> operator-(cx<T> a) { return cx<T>(-a.re, -a.im); }
template <typename T>
FRG_HD cx<T> operator*(cx<T> a, cx<T> b) {
  return cx<T>(fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re));
}
template <typename T>
FRG_HD cx<T> operator*(T s, cx<T> a) { return cx<T>(s * a.re, s * a.im); }
template <typename T>
FRG_HD cx<T> operator*(cx<T> a, T s) { return cx<T>(s * a.re, s * a.im); }
template <typename T>
FRG_HD cx<T>& operator+=(cx<T>& a, cx<T> b) { a.re += b.re; a.im += b.im; return a; }
template <typename T>
FRG_HD cx<T>& operator-=(cx<T>& a, cx<T> b) { a.re -= b.re; a.im -= b.im; return a; }

// a - b*c (one complex fused multiply-subtract: 4 FMA)
template <typename T>
FRG_HD cx<T> cfms(cx<T> a, cx<T> b, cx<T> c) {
  return cx<T>(fma(b.im, c.im, fma(-b.re, c.re, a.re)), fma(-b.im, c.re, fma(-b.re, c.im, a.im)));
}
// a + b*c
template <typename T>
FRG_HD cx<T> cfma(cx<T> b, cx<T> c, cx<T> a) {
  return cx<T>(fma(-b.im, c.im, fma(b.re, c.re, a.re)), fma(b.im, c.re, fma(b.re, c.im, a.im)));
}

template <typename T>
FRG_HD T cnorm2(cx<T> a) { return a.re * a.re + a.im * a.im; }

template <typename T>
FRG_HD T tabs(T x) { return x < T(0) ? -x : x; }

// Smith's division a / b.
template <typename T>
FRG_HD cx<T> cdiv(cx<T> a, cx<T> b) {
  if (tabs(b.re) >= tabs(b.im)) {
    T r = b.im / b.re, d = b.re + b.im * r, id = T(1) / d;
    return cx<T>((a.re + a.im * r) * id, (a.im - a.re * r) * id);
  } else {
    T r = b.re / b.im, d = b.re * r + b.im, id = T(1) / d;
    return cx<T>((a.re * r + a.im) * id, (a.im * r - a.re) * id);
  }
}

// Smith's reciprocal 1 / b.
template <typename T>
FRG_HD cx<T> cinv(cx<T> b) {
  if (tabs(b.re) >= tabs(b.im)) {
    T r = b.im / b.re, id = T(1) / (b.re + b.im * r);
    return cx<T>(id, -r * id);
  } else {
    T r = b.re / b.im, id = T(1) / (b.re * r + b.im);
    return cx<T>(r * id, -id);
  }
}

// FP64: 1/b = conj(b) / |b|^2 with one reciprocal. The tracker's FP64 operands are
// far inside the range where |b|^2 neither overflows nor underflows, so Smith's
// scaling (two divisions) buys nothing there; FP32 keeps Smith's form.
FRG_HD cx<double> cinv(cx<double> b) {
  const double r = 1.0 / (b.re * b.re + b.im * b.im);
  return cx<double>(b.re * r, -b.im * r);
}
FRG_HD cx<double> cdiv(cx<double> a, cx<double> b) { return a * cinv(b); }

