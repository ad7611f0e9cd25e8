// Device building blocks of the path tracker, templated on the working real type.
//
// Layout conventions: complex values are cx<T>; a path state Y is 23 complex
// [Z (21 unknowns), Z0 (homogenizer), t] (htpytrack.cu:46-50); parameters q are 30
// complex [P0..P7, Pc0..Pc7, Q1..Q7, Qc1..Qc7] (htpykinematics.cu:29-33).
#pragma once

#include <stdint.h>

#include "frg_complex.cuh"
#include "frg_rng.h"
#include "frg_system_gen.cuh"

namespace frg {

constexpr int NV = 21;  // unknowns
constexpr int NZ = 22;  // homogeneous unknowns
constexpr int NY = 23;  // path state
constexpr int NP = 30;  // parameters
constexpr int LDM = 24; // leading dimension of the 23x23 system (+ right-hand side)

typedef cx<double> cd;

// Dormand-Prince 6(5) tableau (rungekutta.cu:40-122): stage weights (:40-95), error
// weights (LTE, :99-105) and 6th-order solution weights (:115-122).
static __constant__ double c_dpA[8][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {1. / 10., 0, 0, 0, 0, 0, 0},
    {-2. / 81., 20. / 81., 0, 0, 0, 0, 0},
    {615. / 1372., -270. / 343., 1053. / 1372., 0, 0, 0, 0},
    {3243. / 5500., -54. / 55., 50949. / 71500., 4998. / 17875., 0, 0, 0},
    {-26492. / 37125., 72. / 55., 2808. / 23375., -24206. / 37125., 338. / 459., 0, 0},
    {5561. / 2376., -35. / 11., -24117. / 31603., 899983. / 200772., -5225. / 1836., 3925. / 4056., 0},
    {465467. / 266112., -2945. / 1232., -5610201. / 14158144., 10513573. / 3212352., -424325. / 205632.,
     376225. / 454272., 0}};
static __constant__ double c_dpE[8] = {-13. / 2400., 0., 19683. / 618800., -2401. / 31200., 65. / 816.,
                                -15. / 416., -521. / 5600., 1. / 10.};
static __constant__ double c_dpB[8] = {61. / 864., 0., 98415. / 321776., 16807. / 146016., 1375. / 7344.,
                                1375. / 5408., -37. / 1120., 1. / 10.};


// ---------------------------------------------------------------------------
// Random draws (the reference's curand_uniform_double, replaced by Philox).
// ---------------------------------------------------------------------------
struct Rng {
  uint64_t seed, stream, index;
  __device__ __forceinline__ double uniform() { return frg_uniform01(seed, stream, index++); }
};

// ---------------------------------------------------------------------------
// Start system: a random mechanism and its exact configuration
// (GenerateStart, frgkinematics.cu:13-136).
// ---------------------------------------------------------------------------
__device__ __forceinline__ cd csqrt_halfangle(cd x) {
  // cplxSqrt (classes.cuh:39-45)
  double r = sqrt(x.re * x.re + x.im * x.im);
  double cosA = x.re / r;
  cd out(sqrt(r * (cosA + 1.0) * 0.5), sqrt(r * (1.0 - cosA) * 0.5));
  if (signbit(x.im)) out.im = -out.im;
  return out;
}

__device__ __forceinline__ double start_value(Rng& r, int dist, double range) {
  if (dist == 0) return 2.0 * range * r.uniform() - range;
  double u1 = r.uniform(), u2 = r.uniform();  // Box-Muller, one N(0, 1/2) component
  return sqrt(-log(u1)) * cospi(2.0 * u2);
}

__device__ inline void generate_start(Rng& rng, int dist, double range, cd* z /*21*/, cd* q /*30*/) {
  for (int i = 0; i < 14; ++i) {
    double re = start_value(rng, dist, range);
    double im = start_value(rng, dist, range);
    z[i] = cd(re, im);
  }
  cd P0, Pc0, R[8];
  { double re = start_value(rng, dist, range), im = start_value(rng, dist, range); P0 = cd(re, im); }
  { double re = start_value(rng, dist, range), im = start_value(rng, dist, range); Pc0 = cd(re, im); }
  for (int j = 1; j <= 7; ++j) {
    double re = start_value(rng, dist, range), im = start_value(rng, dist, range);
    R[j] = cd(re, im);
  }
  const cd A = z[0], B = z[1], C = z[2], D = z[3], F = z[4], G = z[5], H = z[6];
  const cd Ac = z[7], Bc = z[8], Cc = z[9], Dc = z[10], Fc = z[11], Gc = z[12], Hc = z[13];
  q[0] = P0;
  q[8] = Pc0;
#pragma unroll 1
  for (int j = 1; j <= 7; ++j) {
    const cd Rj = R[j], iR = cinv(Rj);
    // quadratic in TUc (frgkinematics.cu:63-80)
    cd Aq = (G - D) * (iR * (Hc - Gc) - (Hc - Fc));
    cd Acq = (Gc - Dc) * (Rj * (H - G) - (H - F));
    cd Bq = (-(Rj * ((H - G) * (Hc - Fc))) - iR * ((Hc - Gc) * (H - F))) +
            ((G - D) * (Gc - Dc) + ((H - G) * (Hc - Gc) + ((H - F) * (Hc - Fc) - (F - D) * (Fc - Dc))));
    double pm = rng.uniform() < 0.5 ? -1.0 : 1.0;
    cd disc = csqrt_halfangle(Bq * Bq - 4.0 * (Aq * Acq));
    cd TUc = cinv(2.0 * Aq) * (-Bq + pm * disc);
    cd SUc = cinv(F - D) * (TUc * (G - D) + (Rj * (H - G) - (H - F)));
    // quadratic in U_j (frgkinematics.cu:87-107)
    cd w = (Rj * (H - C) - SUc * (F - B)) - (H - F);
    cd wc = (iR * (Hc - Cc) - cinv(SUc) * (Fc - Bc)) - (Hc - Fc);
    Aq = (Ac - Bc) * w;
    Acq = (A - B) * wc;
    Bq = w * wc + ((A - B) * (Ac - Bc) - (C - A) * (Cc - Ac));
    pm = rng.uniform() < 0.5 ? -1.0 : 1.0;
    disc = csqrt_halfangle(Bq * Bq - 4.0 * (Aq * Acq));
    cd Uj = cinv(2.0 * Aq) * (-Bq + pm * disc);
    z[13 + j] = Uj;
    // rotations and precision points (frgkinematics.cu:109-120)
    cd QUc = cdiv(cd(-1.0), C - A) * (cinv(Uj) * (A - B) + w);
    cd Qj = QUc * Uj;
    q[15 + j] = Qj;
    q[22 + j] = cinv(Qj);
    cd S = SUc * Uj;
    q[j] = B + (S * (F - B) + Uj * (P0 - F));
    q[8 + j] = Bc + (cinv(S) * (Fc - Bc) + cinv(Uj) * (Pc0 - Fc));
  }
}

// ---------------------------------------------------------------------------
// Parameter homotopy q(t) and dq/dt (htpysupport.cu:37-62).
// ---------------------------------------------------------------------------
template <typename T, int N_P = NP>
__device__ __forceinline__ void params_at(T t, const cx<T>* spm, const cx<T>* fpm, cx<T> gamma, cx<T>* q,
                                          cx<T>* dq) {
  const cx<T> g1t = gamma * (T(1) - t);
  const cx<T> iden = cinv(g1t + cx<T>(t));
  const cx<T> gid2 = gamma * (iden * iden);
#pragma unroll 2
  for (int i = 0; i < N_P; ++i) {
    const cx<T> s = spm[i], f = fpm[i];
    q[i] = (g1t * s + t * f) * iden;
    dq[i] = (f - s) * gid2;
  }
}

// ---------------------------------------------------------------------------
// Rows 0..20 of JH and F at Y (htpysupport.cu:89-144, FSYS/JVAR/JPAR):
// row r, columns 0..21 = dF_r/dZ, column 22 = dF_r/dt. Writes full rows into M
// (leading dimension LDM) and F into F[0..20] when F != nullptr.
// ---------------------------------------------------------------------------
template <typename T>
__device__ void system_rows(const cx<T>* Y, const cx<T>* q, const cx<T>* dq, cx<T>* M, cx<T>* Fout) {
  const cx<T> A = Y[0], B = Y[1], C = Y[2], D = Y[3], F = Y[4], G = Y[5], H = Y[6];
  const cx<T> Ac = Y[7], Bc = Y[8], Cc = Y[9], Dc = Y[10], Fc = Y[11], Gc = Y[12], Hc = Y[13];
  const cx<T> z = Y[21];
  const cx<T> e1 = cinv(F - B), e2 = cinv(H - C), ec1 = cinv(Fc - Bc), ec2 = cinv(Hc - Cc);
  const cx<T> z2 = z * z, z3 = z2 * z;
  const cx<T> P0 = q[0], Pc0 = q[8], dP0 = dq[0], dPc0 = dq[8];
  const cx<T> zero(T(0));
#pragma unroll 1
  for (int j = 1; j <= 7; ++j) {
    const cx<T> U = Y[13 + j];
    FrgGroupOut<T> o;
    frg_group_eval<T>(A, B, C, D, F, G, H, Ac, Bc, Cc, Dc, Fc, Gc, Hc, z, e1, e2, ec1, ec2, z2, z3, P0, Pc0,
                      dP0, dPc0, U, cinv(U), q[j], q[8 + j], q[15 + j], q[22 + j], dq[j], dq[8 + j],
                      dq[15 + j], dq[22 + j], o);
    cx<T>* rI = M + (j - 1) * LDM;
    cx<T>* rII = M + (j + 6) * LDM;
    cx<T>* rIII = M + (j + 13) * LDM;
    // family I: {A,C,H,Ac,Cc,Hc,U_j,Z0}
    rI[0] = o.dI[0]; rI[1] = zero; rI[2] = o.dI[1]; rI[3] = zero; rI[4] = zero; rI[5] = zero;
    rI[6] = o.dI[2]; rI[7] = o.dI[3]; rI[8] = zero; rI[9] = o.dI[4]; rI[10] = zero; rI[11] = zero;
    rI[12] = zero; rI[13] = o.dI[5];
    // family II: {B,F,Bc,Fc,U_j,Z0}
    rII[0] = zero; rII[1] = o.dII[0]; rII[2] = zero; rII[3] = zero; rII[4] = o.dII[1]; rII[5] = zero;
    rII[6] = zero; rII[7] = zero; rII[8] = o.dII[2]; rII[9] = zero; rII[10] = zero; rII[11] = o.dII[3];
    rII[12] = zero; rII[13] = zero;
    // family III: {A..H, Ac..Hc, U_j, Z0}
#pragma unroll
    for (int c = 0; c < 14; ++c) rIII[c] = o.dIII[c];
#pragma unroll
    for (int c = 14; c < 21; ++c) { rI[c] = zero; rII[c] = zero; rIII[c] = zero; }
    rI[13 + j] = o.dI[6];
    rII[13 + j] = o.dII[4];
    rIII[13 + j] = o.dIII[14];
    rI[21] = o.dI[7]; rII[21] = o.dII[5]; rIII[21] = o.dIII[15];
    rI[22] = o.tI; rII[22] = o.tII; rIII[22] = o.tIII;
    if (Fout) { Fout[j - 1] = o.fI; Fout[j + 6] = o.fII; Fout[j + 13] = o.fIII; }
  }
}

// Scale rows [0, rows) of M (N_Y columns, leading dimension LD) and, if given, rhs
// by 1/max(|re|,|im|) of the row (htpysupport.cu:259-277, :446-471).
template <typename T, int N_Y = NY, int LD = LDM>
__device__ __forceinline__ void row_scale(cx<T>* M, int rows, cx<T>* rhs) {
#pragma unroll 1
  for (int i = 0; i < rows; ++i) {
    cx<T>* r = M + i * LD;
    T mx = T(0);
#pragma unroll
    for (int c = 0; c < N_Y; ++c) mx = fmax(mx, fmax(tabs(r[c].re), tabs(r[c].im)));
    const T s = T(1) / mx;
#pragma unroll
    for (int c = 0; c < N_Y; ++c) r[c] = s * r[c];
    if (rhs) rhs[i] = s * rhs[i];
  }
}

// Gaussian elimination with partial pivoting on |a|^2 (first maximum wins) over
// rows [0, nelim), right-hand side b, then back substitution
// (LinearSolve, htpysupport.cu:146-232; with nelim = 22 and x[22] = xlast fixed,
// LinearSolveNewton, htpysupport.cu:302-400). Returns the pivot ratio
// max|u_ii| / min|u_ii| over the eliminated rows as a condition estimate. N_Y x N_Y
// with leading dimension LD (23 x 23 and 24 for Stephenson II).
template <typename T, int N_Y = NY, int LD = LDM>
__device__ T lu_solve(cx<T>* M, cx<T>* b, cx<T>* x, int nelim, bool fix_last, cx<T> xlast) {
  T pmax = T(0), pmin = T(-1);  // pmin < 0: no pivot seen yet
  cx<T> ipiv[N_Y];
#pragma unroll 1
  for (int i = 0; i < N_Y; ++i) {
    if (i < nelim) {
      T best = T(0);
      int br = i;
#pragma unroll 1
      for (int k = i; k < nelim; ++k) {
        T v = cnorm2(M[k * LD + i]);
        if (v > best) { best = v; br = k; }
      }
      if (br != i) {
        cx<T>* ri = M + i * LD;
        cx<T>* rb = M + br * LD;
#pragma unroll 1
        for (int c = i; c < N_Y; ++c) { cx<T> tmp = ri[c]; ri[c] = rb[c]; rb[c] = tmp; }
        cx<T> tb = b[i]; b[i] = b[br]; b[br] = tb;
      }
    }
    const cx<T>* ri = M + i * LD;
    const cx<T> ip = cinv(ri[i]);
    ipiv[i] = ip;
    if (i < nelim) {
      T a = sqrt(cnorm2(ri[i]));
      pmax = fmax(pmax, a);
      pmin = (pmin < T(0)) ? a : fmin(pmin, a);
    }
    const cx<T> bi = b[i];
#pragma unroll 1
    for (int j = i + 1; j < nelim; ++j) {
      cx<T>* rj = M + j * LD;
      const cx<T> l = rj[i] * ip;
#pragma unroll 4
      for (int c = i + 1; c < N_Y; ++c) rj[c] = cfms(rj[c], ri[c], l);
      b[j] = cfms(b[j], bi, l);
    }
  }
  int top = N_Y - 1;
  if (fix_last) { x[N_Y - 1] = xlast; top = N_Y - 2; }
#pragma unroll 1
  for (int i = top; i >= 0; --i) {
    const cx<T>* ri = M + i * LD;
    cx<T> sum(T(0));
#pragma unroll 4
    for (int c = i + 1; c < N_Y; ++c) sum = cfma(ri[c], x[c], sum);
    x[i] = ipiv[i] * (b[i] - sum);
  }
  return pmin > T(0) ? pmax / pmin : T(1e30);
}

// SwitchPatch: rescale [Z, Z0] so that unew . [Z, Z0, t] = 1 (htpysupport.cu:9-34);
// N_Y = the path state's length (homogeneous unknowns + t).
template <typename T, int N_Y = NY>
__device__ __forceinline__ void switch_patch(const cx<T>* u, const cx<T>* Yold, cx<T>* Ynew) {
  cx<T> den(T(0));
#pragma unroll 1
  for (int i = 0; i < N_Y - 1; ++i) den = cfma(u[i], Yold[i], den);
  const cx<T> t = Yold[N_Y - 1];
  const cx<T> s = cdiv(cx<T>(T(1)) - u[N_Y - 1] * t, den);
#pragma unroll 1
  for (int i = 0; i < N_Y - 1; ++i) Ynew[i] = s * Yold[i];
  Ynew[N_Y - 1] = t;
}

// Solve the small dense system A x = b (N x N, row-major; A and b are overwritten) by
// Gaussian elimination with partial pivoting on |a|^2, the first maximum winning: the
// plug-in systems' start generation, which solves for the parameters that make a
// random point an exact root.
template <int N>
__device__ __forceinline__ void small_solve(cd* A, cd* b, cd* x) {
#pragma unroll 1
  for (int i = 0; i < N; ++i) {
    int br = i;
    double best = cnorm2(A[i * N + i]);
#pragma unroll 1
    for (int k = i + 1; k < N; ++k) {
      const double v = cnorm2(A[k * N + i]);
      if (v > best) { best = v; br = k; }
    }
    if (br != i) {
#pragma unroll 1
      for (int c = 0; c < N; ++c) { const cd t = A[i * N + c]; A[i * N + c] = A[br * N + c]; A[br * N + c] = t; }
      const cd t = b[i]; b[i] = b[br]; b[br] = t;
    }
#pragma unroll 1
    for (int j = i + 1; j < N; ++j) {
      const cd l = cdiv(A[j * N + i], A[i * N + i]);
#pragma unroll 1
      for (int c = i + 1; c < N; ++c) A[j * N + c] = A[j * N + c] - l * A[i * N + c];
      b[j] = b[j] - l * b[i];
    }
  }
#pragma unroll 1
  for (int i = N - 1; i >= 0; --i) {
    cd sum = b[i];
#pragma unroll 1
    for (int c = i + 1; c < N; ++c) sum = sum - A[i * N + c] * x[c];
    x[i] = cdiv(sum, A[i * N + i]);
  }
}

// ---------------------------------------------------------------------------
// Cognates (Cognate12 and CognateSolns, frgkinematics.cu:185-285).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cognate12(const cd* o, cd P, cd* out) {
  const cd A = o[0], B = o[1], C = o[2], D = o[3], F = o[4], G = o[5], H = o[6];
  cd sc = cdiv(B - F, D - F);
  const cd Dp = sc * (D - H) + H;
  const cd Gp = sc * (G - H) + H;
  sc = cdiv(P - F, H - F);
  out[0] = sc * (A - B) + B;
  out[1] = B;
  out[2] = sc * (C - B) + B;
  out[3] = sc * (Dp - B) + B;
  out[4] = B + (P - F);
  out[5] = sc * (Gp - B) + B;
  out[6] = sc * (H - B) + B;
}

// root (21) -> canonical of {root, 1/2 cognate}: the one with the smaller Re(A).
__device__ inline void canonical_cognate(const cd* r0, const cd* fpm, cd* out) {
  cd r1[NV];
  const cd B = r0[1], F = r0[4], P0 = fpm[0], Pc0 = fpm[8];
  const cd iFB = cinv(F - B);
#pragma unroll 1
  for (int i = 1; i <= 7; ++i) r1[13 + i] = ((fpm[i] - B) - r0[13 + i] * (P0 - F)) * iFB;
  cognate12(r0, P0, r1);
  cognate12(r0 + 7, Pc0, r1 + 7);
  const bool swap = r1[0].re < r0[0].re;
#pragma unroll 1
  for (int i = 0; i < NV; ++i) out[i] = swap ? r1[i] : r0[i];
}

// The Stephenson II system as the tracker's system type (the other systems are the
// generated plug-ins of frg_plugins_gen.cuh, with the same members): rows of the
// homotopy Jacobian and F, the start (GenerateStart), the canonical root (cognates).
struct SysStephenson2 {
  static constexpr int ID = 0;
  static constexpr int NV = frg::NV;
  static constexpr int NP = frg::NP;
  template <typename T, int LD>
  __device__ static void rows(const cx<T>* Y, const cx<T>* q, const cx<T>* dq, cx<T>* M, cx<T>* F) {
    static_assert(LD == LDM, "Stephenson II rows are laid out with leading dimension LDM");
    system_rows<T>(Y, q, dq, M, F);
  }
  __device__ static void start(Rng& rng, int dist, double range, cd* z, cd* q) {
    generate_start(rng, dist, range, z, q);
  }
  __device__ static void canonical(const cd* root, const cd* fpm, cd* out) { canonical_cognate(root, fpm, out); }
};

}  // namespace frg
