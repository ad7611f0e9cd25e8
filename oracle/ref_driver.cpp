/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * Host driver for the reference tracker's own sources, compiled unchanged for the
 * CPU by oracle/Makefile (g++, with oracle/ref_stub/curand_kernel.h first on the
 * include path). It exposes the reference's hot-path functions through a plain C
 * ABI so that tests/golden/make_golden.py can record golden vectors and the
 * C restatement (frg_oracle.c) can be pinned against them.
 *
 * Each wrapper calls exactly one reference function; ref_homotopy_path restates
 * the four calls of the reference kernel body (frg.cu:41-68) for one path.
 * Complex arrays are interleaved (re, im) doubles, the byte layout of the
 * reference's Vect<M>/Matr<R,C> (classes.cuh:52-54, 136-139).
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "htpysupport.cuh"
#include "rungekutta.cuh"
#include "htpytrack.cuh"
#include "frgkinematics.cuh"
#include "frgsupport.cuh"

template <int M>
static void load(Vect<M>* v, const double* src) { std::memcpy(v->vals, src, sizeof(Cplx) * M); }
template <int M>
static void store(const Vect<M>* v, double* dst) { std::memcpy(dst, v->vals, sizeof(Cplx) * M); }

extern "C" {

/* FSYS (htpykinematics.cu:8): Z = 22 complex (21 unknowns + homogenizer), q = 30 complex. */
void ref_fsys(const double* Z, const double* q, double* out) {
  Vect<nV + 1> z; Vect<nP> p; Vect<nV> f;
  load(&z, Z); load(&p, q);
  FSYS(&z, &p, &f);
  store(&f, out);
}

/* JVAR (htpykinematics.cu:129): 21 x 22 row-major. */
void ref_jvar(const double* Z, const double* q, double* out) {
  Vect<nV + 1> z; Vect<nP> p; Matr<nV, nV + 1> m;
  load(&z, Z); load(&p, q);
  JVAR(&z, &p, &m);
  std::memcpy(out, m.vals, sizeof(m.vals));
}

/* JPAR (htpykinematics.cu:1132): 21 x 30 row-major. */
void ref_jpar(const double* Z, const double* q, double* out) {
  Vect<nV + 1> z; Vect<nP> p; Matr<nV, nP> m;
  load(&z, Z); load(&p, q);
  JPAR(&z, &p, &m);
  std::memcpy(out, m.vals, sizeof(m.vals));
}

/* q(t) and dq/dt (htpysupport.cu:37, :51). */
void ref_q(double t, const double* spm, const double* fpm, const double* gamma, double* out) {
  Vect<nP> s, f, o; Cplx g = {gamma[0], gamma[1]};
  load(&s, spm); load(&f, fpm);
  q(t, &s, &f, &g, &o);
  store(&o, out);
}
void ref_dqdt(double t, const double* spm, const double* fpm, const double* gamma, double* out) {
  Vect<nP> s, f, o; Cplx g = {gamma[0], gamma[1]};
  load(&s, spm); load(&f, fpm);
  dqdt(t, &s, &f, &g, &o);
  store(&o, out);
}

/* H (htpysupport.cu:64): 22 complex. */
void ref_h(const double* Y, const double* u, const double* spm, const double* fpm,
           const double* gamma, double* out) {
  Vect<nV + 2> y, uu; Vect<nP> s, f; Vect<nV + 1> h; Cplx g = {gamma[0], gamma[1]};
  load(&y, Y); load(&uu, u); load(&s, spm); load(&f, fpm);
  H(&y, &uu, &s, &f, &g, &h);
  store(&h, out);
}

/* JH (htpysupport.cu:89): 22 x 23 row-major. */
void ref_jh(const double* Y, const double* u, const double* spm, const double* fpm,
            const double* gamma, double* out) {
  Vect<nV + 2> y, uu; Vect<nP> s, f; Matr<nV + 2, nV + 2> m; Cplx g = {gamma[0], gamma[1]};
  load(&y, Y); load(&uu, u); load(&s, spm); load(&f, fpm);
  JH(&y, &uu, &s, &f, &g, (Matr<nV + 1, nV + 2>*)&m);
  std::memcpy(out, m.vals, sizeof(Cplx) * (nV + 1) * (nV + 2));
}

/* SwitchPatch (htpysupport.cu:9). */
void ref_switch_patch(const double* u, const double* Yold, double* Ynew) {
  Vect<nV + 2> uu, yo, yn;
  load(&uu, u); load(&yo, Yold);
  SwitchPatch(&uu, &yo, &yn);
  store(&yn, Ynew);
}

/* IVP (htpysupport.cu:237): tangent at Yc with velocity patch Vc. */
void ref_ivp(int tstepQ, const double* Yc, const double* Vc, const double* u, const double* spm,
             const double* fpm, const double* gamma, double* out) {
  Vect<nV + 2> y, v, uu, o; Vect<nP> s, f; Cplx g = {gamma[0], gamma[1]};
  load(&y, Yc); load(&v, Vc); load(&uu, u); load(&s, spm); load(&f, fpm);
  IVP(tstepQ != 0, &y, &v, &uu, &s, &f, &g, &o);
  store(&o, out);
}

/* DormandPrince65 (rungekutta.cu:3): one predictor attempt. */
void ref_dp65(double step, double tol, int tstepQ, const double* Yc, const double* Vc,
              const double* u, const double* spm, const double* fpm, const double* gamma,
              double* Yn, double* Vn, double* err, double* scale) {
  Vect<nV + 2> y, v, uu, yn, vn; Vect<nP> s, f; Cplx g = {gamma[0], gamma[1]};
  load(&y, Yc); load(&v, Vc); load(&uu, u); load(&s, spm); load(&f, fpm);
  DormandPrince65(step, tol, tstepQ != 0, &y, &v, &uu, &s, &f, &g, &yn, &vn, err, scale);
  store(&yn, Yn); store(&vn, Vn);
}

/* Newton (htpysupport.cu:407): YN is input start point and output. */
void ref_newton(double tgoal, const double* Vn, const double* u, const double* spm,
                const double* fpm, const double* gamma, int maxIts, double tol, int residualtype,
                double* YN, double* residual) {
  Vect<nV + 2> v, uu, y; Vect<nP> s, f; Cplx g = {gamma[0], gamma[1]};
  load(&v, Vn); load(&uu, u); load(&s, spm); load(&f, fpm); load(&y, YN);
  Newton(tgoal, &v, &uu, &s, &f, &g, maxIts, tol, residualtype, &y, residual);
  store(&y, YN);
}

/* GenerateStart (frgkinematics.cu:13) on stream `stream` of `seed`. */
void ref_generate_start(unsigned long long seed, unsigned long long stream, double* spt, double* spm) {
  curandState st; curand_init(seed, stream, 0, &st);
  Vect<nV> z; Vect<nP> q;
  GenerateStart(st, &z, &q);
  store(&z, spt); store(&q, spm);
}

/* TrackPath (htpytrack.cu:33) from an explicit start; the RNG state it receives is
   the fresh state of `stream`, as in the reference kernel (frg.cu:54,57). */
void ref_track_path(const double* spt, const double* spm, const double* fpm, const double* gamma,
                    unsigned long long seed, unsigned long long stream, double* Yfinal, int* code) {
  curandState st; curand_init(seed, stream, 0, &st);
  Vect<nV + 2> yf; Vect<nP> s, f; Cplx g = {gamma[0], gamma[1]};
  Vect<nV>* z = (Vect<nV>*)&yf;
  std::memcpy(z->vals, spt, sizeof(Cplx) * nV);
  load(&s, spm); load(&f, fpm);
  TrackPath(z, &s, &f, &g, st, &yf, code);
  store(&yf, Yfinal);
}

/* CognateSolns (frgkinematics.cu:227): out = 2 x 21, canonical root first. */
void ref_cognate(const double* z, const double* q, double* out) {
  Vect<nV> c[2]; Vect<nP> p;
  load(&c[0], z); load(&p, q);
  CognateSolns(&c[0], &p, c);
  store(&c[0], out); store(&c[1], out + 2 * nV);
}

/* The reference kernel body for one path (frg.cu:41-68): start, track,
   dehomogenize, canonical cognate. Yfinal (23 complex, before dehomogenizing) is
   also returned. */
void ref_homotopy_path(unsigned long long seed, unsigned long long stream, const double* fpm,
                       const double* gamma, double* root, int* code, double* Yfinal_out) {
  curandState st; curand_init(seed, stream, 0, &st);
  Cplx g = {gamma[0], gamma[1]};
  Vect<nV + 2> u_dehom;
  std::memset(u_dehom.vals, 0, sizeof(Vect<nV + 2>));
  u_dehom.vals[nV] = {1., 0};
  Vect<nV + 2> Yfinal;
  Vect<nV>* spt = (Vect<nV>*)&Yfinal;
  Vect<nP> spm, f;
  load(&f, fpm);
  GenerateStart(st, spt, &spm);
  TrackPath(spt, &spm, &f, &g, st, &Yfinal, code);
  if (Yfinal_out) store(&Yfinal, Yfinal_out);
  SwitchPatch(&u_dehom, &Yfinal, &Yfinal);
  Vect<nV> cogn[2];
  cogn[0].set(Yfinal.vals);
  CognateSolns(&cogn[0], &f, cogn);
  store(&cogn[0], root);
}

/* A batch of paths on `nthreads` host threads, streams stream0 .. stream0+n-1. */
void ref_homotopy_batch(unsigned long long seed, unsigned long long stream0, long long n,
                        const double* fpm, const double* gamma, double* roots, int* codes,
                        int nthreads) {
  if (nthreads < 1) nthreads = 1;
  std::vector<std::thread> pool;
  for (int w = 0; w < nthreads; ++w) {
    pool.emplace_back([=]() {
      for (long long i = w; i < n; i += nthreads)
        ref_homotopy_path(seed, stream0 + (unsigned long long)i, fpm, gamma, roots + 2 * nV * i,
                          codes + i, nullptr);
    });
  }
  for (auto& t : pool) t.join();
}

/* Row-scaled residual of the target system at a dehomogenized root (Z0 = 1):
   max over the 21 rows of |F_r| / max_c max(|Re J_rc|, |Im J_rc|), with FSYS and JVAR
   (htpykinematics.cu:8, :129) -- the residual the GPU tracker reports per root. */
static double root_residual(const Vect<nV>* root, const Vect<nP>* q) {
  Vect<nV + 1> z; Vect<nP> p = *q; Vect<nV> f; Matr<nV, nV + 1> m;
  std::memcpy(z.vals, root->vals, sizeof(Cplx) * nV);
  z.vals[nV] = {1.0, 0.0};
  FSYS(&z, &p, &f);
  JVAR(&z, &p, &m);
  double r = 0.0;
  for (int i = 0; i < nV; ++i) {
    double mx = 0.0;
    for (int c = 0; c < nV + 1; ++c) {
      const Cplx v = m.vals[i * (nV + 1) + c];
      mx = std::max(mx, std::max(std::fabs(v.x), std::fabs(v.y)));
    }
    const double fr = std::sqrt(f.vals[i].x * f.vals[i].x + f.vals[i].y * f.vals[i].y);
    const double ri = fr / mx;
    r = (ri == ri) ? std::max(r, ri) : INFINITY;  /* a non-finite row: infinite residual */
  }
  return r;
}

/* The reference kernel body for one path (frg.cu:41-68) with the start mechanism drawn
   either as the reference draws it (start_normal = 0: U(-5,5)^2, frgkinematics.cu:7-8)
   or complex normal (start_normal = 1, through the stub's mode 1); TrackPath gets the
   fresh state by value as in frg.cu:54,57. Also returns Yfinal (23 complex) and the
   root's residual. */
void ref_homotopy_path_ex(unsigned long long seed, unsigned long long stream, const double* fpm,
                          const double* gamma, int start_normal, double* root, int* code, double* Yfinal_out,
                          double* resid) {
  curandState st; curand_init(seed, stream, 0, &st);
  curandState st_start = st;
  st_start.mode = start_normal ? 1 : 0;
  Cplx g = {gamma[0], gamma[1]};
  Vect<nV + 2> u_dehom;
  std::memset(u_dehom.vals, 0, sizeof(Vect<nV + 2>));
  u_dehom.vals[nV] = {1., 0};
  Vect<nV + 2> Yfinal;
  Vect<nV>* spt = (Vect<nV>*)&Yfinal;
  Vect<nP> spm, f;
  load(&f, fpm);
  GenerateStart(st_start, spt, &spm);
  TrackPath(spt, &spm, &f, &g, st, &Yfinal, code);
  if (Yfinal_out) store(&Yfinal, Yfinal_out);
  SwitchPatch(&u_dehom, &Yfinal, &Yfinal);
  Vect<nV> cogn[2];
  cogn[0].set(Yfinal.vals);
  CognateSolns(&cogn[0], &f, cogn);
  store(&cogn[0], root);
  if (resid) *resid = root_residual(&cogn[0], &f);
}

/* A batch of ref_homotopy_path_ex on `nthreads` host threads, streams stream0 ..
   stream0 + n - 1 (yfinal and resid optional). */
void ref_homotopy_batch_ex(unsigned long long seed, unsigned long long stream0, long long n, const double* fpm,
                           const double* gamma, int start_normal, double* roots, int* codes, double* yfinal,
                           double* resid, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  std::vector<std::thread> pool;
  for (int w = 0; w < nthreads; ++w) {
    pool.emplace_back([=]() {
      for (long long i = w; i < n; i += nthreads)
        ref_homotopy_path_ex(seed, stream0 + (unsigned long long)i, fpm, gamma, start_normal, roots + 2 * nV * i,
                             codes + i, yfinal ? yfinal + 2 * (nV + 2) * i : nullptr, resid ? resid + i : nullptr);
    });
  }
  for (auto& t : pool) t.join();
}

/* root_residual for n dehomogenized roots (n x 21 complex) of the target fpm. */
void ref_residuals(const double* roots, long long n, const double* fpm, double* out) {
  Vect<nP> f;
  load(&f, fpm);
  for (long long i = 0; i < n; ++i) {
    Vect<nV> r;
    load(&r, roots + 2 * nV * i);
    out[i] = root_residual(&r, &f);
  }
}

/* One uniform draw of the shared Philox stream (the stub's generator). */
double ref_uniform01(unsigned long long seed, unsigned long long stream, unsigned long long index) {
  return frg_uniform01(seed, stream, index);
}

/* SortingDeletingMerging (frgsupport.cu:10) on a collection held by the caller.
   coll: ncoll x 21 complex, sorted; coll_out must hold ncoll + n roots; order is
   the index order of fpt by Re(root[0]) (frg.cu:432-435). Returns the new size. */
long long ref_sort_merge(const double* coll, long long ncoll, const double* fpt, int* codes,
                         const int* order, int n, double* coll_out) {
  std::deque<Vect<nV>> dq((size_t)ncoll);
  for (long long i = 0; i < ncoll; ++i) load(&dq[(size_t)i], coll + 2 * nV * i);
  std::vector<Vect<nV>> f((size_t)n);
  for (int i = 0; i < n; ++i) load(&f[(size_t)i], fpt + 2 * nV * i);
  std::vector<int> ord(order, order + n);
  SortingDeletingMerging(&dq, f.data(), codes, ord.data(), n);
  for (size_t i = 0; i < dq.size(); ++i) store(&dq[i], coll_out + 2 * nV * i);
  return (long long)dq.size();
}

/* LambertW (frgsupport.cu:249). */
double ref_lambertw(double z) { return LambertW(z); }

}  // extern "C"
