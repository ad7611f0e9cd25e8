/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * Plain-C restatement of the reference path tracker, the checker for the CUDA
 * kernels. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * it. Every function names the reference file:line it restates. The Jacobians are
 * derived by hand from the loop-closure equations (chain rule through the
 * intermediate quantities below), not transcribed from the reference's JVAR/JPAR;
 * tests pin them against golden vectors recorded from the reference itself.
 *
 * Complex division is Smith's algorithm (R. L. Smith, CACM 5(8), 1962).
 *
 * The tracker (IVP, DP6(5), Newton, TrackPath) takes the system as a parameter (osys):
 * Stephenson II, restated here, or a generated plug-in system (frg_plugins_gen.h, from the
 * sympy modules in finite_root_generation_gb300/systems), which has no reference
 * counterpart; its rows are checked against the symbolic system in tests/.
 */
#define _GNU_SOURCE
#include "frg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../finite_root_generation_gb300/csrc/frg_rng.h"

typedef struct { double re, im; } cd;

static inline cd mk(double re, double im) { cd z; z.re = re; z.im = im; return z; }
static inline cd cadd(cd a, cd b) { return mk(a.re + b.re, a.im + b.im); }
static inline cd csub(cd a, cd b) { return mk(a.re - b.re, a.im - b.im); }
static inline cd cmul(cd a, cd b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cd cscal(double s, cd a) { return mk(s * a.re, s * a.im); }
static inline cd cdiv(cd a, cd b) {
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, d = b.re + b.im * r;
    return mk((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  } else {
    double r = b.re / b.im, d = b.re * r + b.im;
    return mk((a.re * r + a.im) / d, (a.im * r - a.re) / d);
  }
}
static inline cd cinv(cd b) { return cdiv(mk(1.0, 0.0), b); }
static inline double cnorm2(cd a) { return a.re * a.re + a.im * a.im; }
static inline cd ld(const double* p, int i) { return mk(p[2 * i], p[2 * i + 1]); }
static inline void st(double* p, int i, cd z) { p[2 * i] = z.re; p[2 * i + 1] = z.im; }
static inline cd m3(cd a, cd b, cd c) { return cmul(cmul(a, b), c); }

/* cplxSqrt (classes.cuh:39-45): principal root through the half-angle formulas. */
static cd csqrt_ref(cd x) {
  double r = sqrt(cnorm2(x));
  double cosA = x.re / r;
  cd out = mk(sqrt(r * (cosA + 1.0) / 2.0), sqrt(r * (1.0 - cosA) / 2.0));
  if (signbit(x.im)) out.im = -out.im;
  return out;
}

void or_config_default(or_config* c) {
  c->s_init = 1.0; c->s_max = 100.0; c->s_min = 1e-6; c->rk_tol = 1e-3;
  c->caution_steps = 2;
  c->newt_its = 10; c->newt_tol = 1e-8; c->newt_residual = 1; c->newt_attempts = 3;
  c->sharp_its = 30; c->sharp_tol = 1e-12; c->sharp_residual = 1; c->sharp_attempts = 3;
  c->sharp_trigger = 1e-5; c->nudge_trigger = 1e-5;
  c->max_steps = 2000; c->max_ministeps = 3000;
  c->patch_range = 2.0;
  c->start_dist = 0; c->start_range = 5.0;
}

/* ------------------------------------------------------------------------- */
/* The Stephenson II loop-closure system (htpykinematics.cu:8-126).           */
/* ------------------------------------------------------------------------- */

typedef struct {
  cd A, B, C, D, F, G, H, Ac, Bc, Cc, Dc, Fc, Gc, Hc, z;
} links;

static void unpack_links(const double* Z, links* L) {
  L->A = ld(Z, 0); L->B = ld(Z, 1); L->C = ld(Z, 2); L->D = ld(Z, 3);
  L->F = ld(Z, 4); L->G = ld(Z, 5); L->H = ld(Z, 6);
  L->Ac = ld(Z, 7); L->Bc = ld(Z, 8); L->Cc = ld(Z, 9); L->Dc = ld(Z, 10);
  L->Fc = ld(Z, 11); L->Gc = ld(Z, 12); L->Hc = ld(Z, 13);
  L->z = ld(Z, 21);
}

/*
 * Equations j-1, j+6 and j+13 of FSYS for one j (htpykinematics.cu:36-122), with
 * optional derivatives: dZ[r][c] = d(eq r)/d(Z_c) over the 22 unknowns (U_j is
 * column 13+j, Z0 column 21), dq[r][k] = derivative w.r.t. (P0, Pj, Pc0, Pcj, Qj, Qcj).
 *
 * With p = Pj Z0, pc = Pcj Z0, p0 = P0 Z0, pc0 = Pc0 Z0, a = C - A, ac = Cc - Ac:
 *  I  : -S Z0^3 + ac Qc Z0 (p-A) + Ac Z0 (a+p) + Hc Z0 (p0-C) + a Q Z0 (pc-Ac)
 *       + A Z0 (ac+pc) + U (p0-H) m + H Z0 (pc0-Cc) + Z0^2 n (pc0-Hc) / U,
 *       S = Pj Pcj + P0 Pc0, m = pc - Ac - ac Qc, n = p - A - a Q
 *  II : Z0^2 (Bc Pj + B Pcj) - S Z0^3 + Fc Z0 (p0-B) + U (p0-F)(pc-Bc)
 *       + F Z0 (pc0-Bc) + Z0^2 (p-B)(pc0-Fc) / U
 *  III: (G-D)(Gc-Dc) Z0 - Z0 X Xc + U W Xc + Z0^2 X Wc / U - Z0 W Wc,
 *       X = (A-B) + a Q - (D-B)(p-B)/(F-B) + (G-C) n/(H-C),
 *       W = -(D-B)(p0-F)/(F-B) + (G-C)(p0-H)/(H-C), and Xc, Wc their conjugate-side twins.
 */
static void eqs_j(const links* L, const cd U, int j, const double* q, cd f[3], cd dZ[3][22],
                  cd dq[3][6]) {
  const cd z = L->z;
  const cd P0 = ld(q, 0), Pj = ld(q, j), Pc0 = ld(q, 8), Pcj = ld(q, 8 + j);
  const cd Q = ld(q, 15 + j), Qc = ld(q, 22 + j);
  const cd A = L->A, B = L->B, C = L->C, D = L->D, F = L->F, G = L->G, H = L->H;
  const cd Ac = L->Ac, Bc = L->Bc, Cc = L->Cc, Dc = L->Dc, Fc = L->Fc, Gc = L->Gc, Hc = L->Hc;

  const cd z2 = cmul(z, z), z3 = cmul(z2, z);
  const cd p = cmul(Pj, z), pc = cmul(Pcj, z), p0 = cmul(P0, z), pc0 = cmul(Pc0, z);
  const cd a = csub(C, A), ac = csub(Cc, Ac);
  const cd S = cadd(cmul(Pj, Pcj), cmul(P0, Pc0));
  const cd iU = cinv(U), iU2 = cmul(iU, iU);

  /* ---- family I (row j-1) ---- */
  const cd pmA = csub(p, A), pcmAc = csub(pc, Ac), p0mH = csub(p0, H), p0mC = csub(p0, C);
  const cd pc0mHc = csub(pc0, Hc), pc0mCc = csub(pc0, Cc);
  const cd m = csub(pcmAc, cmul(ac, Qc));
  const cd n = csub(pmA, cmul(a, Q));
  {
    cd T1 = cmul(mk(-1, 0), cmul(S, z3));
    cd T2 = cmul(m3(ac, Qc, z), pmA);
    cd T3 = cmul(cmul(Ac, z), cadd(a, p));
    cd T4 = cmul(cmul(Hc, z), p0mC);
    cd T5 = cmul(m3(a, Q, z), pcmAc);
    cd T6 = cmul(cmul(A, z), cadd(ac, pc));
    cd T7 = cmul(cmul(U, p0mH), m);
    cd T8 = cmul(cmul(H, z), pc0mCc);
    cd T9 = cmul(m3(z2, n, pc0mHc), iU);
    f[0] = cadd(cadd(cadd(cadd(cadd(cadd(cadd(cadd(T1, T2), T3), T4), T5), T6), T7), T8), T9);
  }
  /* ---- family II (row j+6) ---- */
  const cd p0mB = csub(p0, B), p0mF = csub(p0, F), pcmBc = csub(pc, Bc), pc0mBc = csub(pc0, Bc);
  const cd pmB = csub(p, B), pc0mFc = csub(pc0, Fc);
  {
    cd T1 = cmul(z2, cadd(cmul(Bc, Pj), cmul(B, Pcj)));
    cd T2 = cmul(S, z3);
    cd T3 = cmul(cmul(Fc, z), p0mB);
    cd T4 = cmul(cmul(U, p0mF), pcmBc);
    cd T5 = cmul(cmul(F, z), pc0mBc);
    cd T6 = cmul(m3(z2, pmB, pc0mFc), iU);
    f[1] = cadd(cadd(cadd(cadd(csub(T1, T2), T3), T4), T5), T6);
  }
  /* ---- family III (row j+13) ---- */
  const cd k1 = csub(D, B), k2 = csub(G, C), e1 = cinv(csub(F, B)), e2 = cinv(csub(H, C));
  const cd kc1 = csub(Dc, Bc), kc2 = csub(Gc, Cc), ec1 = cinv(csub(Fc, Bc)), ec2 = cinv(csub(Hc, Cc));
  const cd nc = m; /* pc - Ac - ac Qc */
  const cd X = cadd(csub(cadd(csub(A, B), cmul(a, Q)), m3(k1, pmB, e1)), m3(k2, n, e2));
  const cd Xc = cadd(csub(cadd(csub(Ac, Bc), cmul(ac, Qc)), m3(kc1, pcmBc, ec1)), m3(kc2, nc, ec2));
  const cd W = cadd(cmul(mk(-1, 0), m3(k1, p0mF, e1)), m3(k2, p0mH, e2));
  const cd p0mFc_c = csub(pc0, Fc), pc0mHc_c = pc0mHc;
  const cd Wc = cadd(cmul(mk(-1, 0), m3(kc1, p0mFc_c, ec1)), m3(kc2, pc0mHc_c, ec2));
  const cd GD = cmul(csub(G, D), csub(Gc, Dc));
  f[2] = csub(cadd(cadd(csub(cmul(GD, z), m3(z, X, Xc)), m3(U, W, Xc)), cmul(m3(z2, X, Wc), iU)),
              m3(z, W, Wc));

  if (!dZ && !dq) return;

  /* ---- derivatives, family I ---- */
  cd* r = dZ ? dZ[0] : NULL;
  const cd Qm1 = csub(Q, mk(1, 0)), Qcm1 = csub(Qc, mk(1, 0));
  if (r) {
    for (int c = 0; c < 22; ++c) r[c] = mk(0, 0);
    r[0] = cadd(cadd(csub(csub(cmul(mk(-1, 0), m3(ac, Qc, z)), cmul(Ac, z)), m3(Q, z, pcmAc)),
                     cmul(z, cadd(ac, pc))),
                m3(z2, pc0mHc, cmul(iU, Qm1)));
    r[2] = csub(cadd(csub(cmul(Ac, z), cmul(Hc, z)), m3(Q, z, pcmAc)), m3(z2, pc0mHc, cmul(iU, Q)));
    r[6] = cadd(cmul(mk(-1, 0), cmul(U, m)), cmul(z, pc0mCc));
    r[7] = cadd(csub(csub(cadd(cmul(mk(-1, 0), m3(Qc, z, pmA)), cmul(z, cadd(a, p))), m3(a, Q, z)),
                     cmul(A, z)),
                m3(U, p0mH, Qcm1));
    r[9] = csub(csub(cadd(m3(Qc, z, pmA), cmul(A, z)), m3(U, p0mH, Qc)), cmul(H, z));
    r[13] = csub(cmul(z, p0mC), m3(z2, n, iU));
    r[13 + j] = csub(cmul(p0mH, m), cmul(m3(z2, n, pc0mHc), iU2));
    {
      cd t = cmul(mk(-3, 0), cmul(S, z2));
      t = cadd(t, m3(ac, Qc, cadd(pmA, cmul(z, Pj))));
      t = cadd(t, cmul(Ac, cadd(cadd(a, p), cmul(z, Pj))));
      t = cadd(t, cmul(Hc, cadd(p0mC, cmul(z, P0))));
      t = cadd(t, m3(a, Q, cadd(pcmAc, cmul(z, Pcj))));
      t = cadd(t, cmul(A, cadd(cadd(ac, pc), cmul(z, Pcj))));
      t = cadd(t, cmul(U, cadd(cmul(P0, m), cmul(p0mH, Pcj))));
      t = cadd(t, cmul(H, cadd(pc0mCc, cmul(z, Pc0))));
      cd u9 = cadd(cadd(cmul(cmul(mk(2, 0), z), cmul(n, pc0mHc)), m3(z2, Pj, pc0mHc)), m3(z2, n, Pc0));
      r[21] = cadd(t, cmul(u9, iU));
    }
  }
  if (dq) {
    cd* g = dq[0];
    g[0] = cadd(csub(cmul(Hc, z2), cmul(Pc0, z3)), m3(U, z, m));
    g[1] = cadd(cadd(csub(m3(ac, Qc, z2), cmul(Pcj, z3)), cmul(Ac, z2)), m3(z3, pc0mHc, iU));
    g[2] = cadd(csub(cmul(H, z2), cmul(P0, z3)), m3(z3, n, iU));
    g[3] = cadd(cadd(csub(m3(a, Q, z2), cmul(Pj, z3)), cmul(A, z2)), m3(U, p0mH, z));
    g[4] = csub(m3(a, z, pcmAc), cmul(m3(z2, a, pc0mHc), iU));
    g[5] = csub(m3(ac, z, pmA), m3(U, p0mH, ac));
  }
  /* ---- derivatives, family II ---- */
  r = dZ ? dZ[1] : NULL;
  if (r) {
    for (int c = 0; c < 22; ++c) r[c] = mk(0, 0);
    r[1] = csub(csub(cmul(Pcj, z2), cmul(Fc, z)), cmul(cmul(z2, pc0mFc), iU));
    r[4] = cadd(cmul(mk(-1, 0), cmul(U, pcmBc)), cmul(z, pc0mBc));
    r[8] = csub(csub(cmul(Pj, z2), cmul(U, p0mF)), cmul(F, z));
    r[11] = csub(cmul(z, p0mB), cmul(cmul(z2, pmB), iU));
    r[13 + j] = csub(cmul(p0mF, pcmBc), cmul(m3(z2, pmB, pc0mFc), iU2));
    {
      cd t = cmul(cmul(mk(2, 0), z), cadd(cmul(Bc, Pj), cmul(B, Pcj)));
      t = csub(t, cmul(mk(3, 0), cmul(S, z2)));
      t = cadd(t, cmul(Fc, cadd(p0mB, cmul(z, P0))));
      t = cadd(t, cmul(U, cadd(cmul(P0, pcmBc), cmul(p0mF, Pcj))));
      t = cadd(t, cmul(F, cadd(pc0mBc, cmul(z, Pc0))));
      cd u6 = cadd(cadd(cmul(cmul(mk(2, 0), z), cmul(pmB, pc0mFc)), m3(z2, Pj, pc0mFc)), m3(z2, pmB, Pc0));
      r[21] = cadd(t, cmul(u6, iU));
    }
  }
  if (dq) {
    cd* g = dq[1];
    g[0] = cadd(csub(cmul(Fc, z2), cmul(Pc0, z3)), m3(U, z, pcmBc));
    g[1] = cadd(csub(cmul(Bc, z2), cmul(Pcj, z3)), m3(z3, pc0mFc, iU));
    g[2] = cadd(csub(cmul(F, z2), cmul(P0, z3)), m3(z3, pmB, iU));
    g[3] = cadd(csub(cmul(B, z2), cmul(Pj, z3)), m3(U, p0mF, z));
    g[4] = mk(0, 0);
    g[5] = mk(0, 0);
  }
  /* ---- derivatives, family III ---- */
  const cd fX = cadd(cmul(mk(-1, 0), cmul(z, Xc)), cmul(cmul(z2, Wc), iU));
  const cd fXc = cadd(cmul(mk(-1, 0), cmul(z, X)), cmul(U, W));
  const cd fW = csub(cmul(U, Xc), cmul(z, Wc));
  const cd fWc = csub(cmul(cmul(z2, X), iU), cmul(z, W));
  const cd one = mk(1, 0);
  const cd k2e2 = cmul(k2, e2), k1e1 = cmul(k1, e1), e1s = cmul(e1, e1), e2s = cmul(e2, e2);
  const cd kc2ec2 = cmul(kc2, ec2), kc1ec1 = cmul(kc1, ec1), ec1s = cmul(ec1, ec1), ec2s = cmul(ec2, ec2);
  const cd slope = csub(k2e2, k1e1), slopec = csub(kc2ec2, kc1ec1);
  /* dX/d(A,B,C,D,F,G,H,z) and dW/d(B,C,D,F,G,H,z) */
  cd XA = cmul(csub(one, Q), csub(one, k2e2));
  cd XB = csub(cadd(cadd(mk(-1, 0), cmul(pmB, e1)), k1e1), m3(k1, pmB, e1s));
  cd XC = cadd(csub(csub(Q, cmul(n, e2)), cmul(k2e2, Q)), m3(k2, n, e2s));
  cd XD = cmul(mk(-1, 0), cmul(pmB, e1));
  cd XF = m3(k1, pmB, e1s);
  cd XG = cmul(n, e2);
  cd XH = cmul(mk(-1, 0), m3(k2, n, e2s));
  cd Xz = cmul(Pj, slope);
  cd WB = csub(cmul(p0mF, e1), m3(k1, p0mF, e1s));
  cd WC = cadd(cmul(mk(-1, 0), cmul(p0mH, e2)), m3(k2, p0mH, e2s));
  cd WD = cmul(mk(-1, 0), cmul(p0mF, e1));
  cd WF = cadd(k1e1, m3(k1, p0mF, e1s));
  cd WG = cmul(p0mH, e2);
  cd WH = csub(cmul(mk(-1, 0), k2e2), m3(k2, p0mH, e2s));
  cd Wz = cmul(P0, slope);
  /* conjugate side */
  const cd pcmBc_ = pcmBc, pc0mFc_ = pc0mFc, pc0mHc_ = pc0mHc;
  cd XcA = cmul(csub(one, Qc), csub(one, kc2ec2));
  cd XcB = csub(cadd(cadd(mk(-1, 0), cmul(pcmBc_, ec1)), kc1ec1), m3(kc1, pcmBc_, ec1s));
  cd XcC = cadd(csub(csub(Qc, cmul(nc, ec2)), cmul(kc2ec2, Qc)), m3(kc2, nc, ec2s));
  cd XcD = cmul(mk(-1, 0), cmul(pcmBc_, ec1));
  cd XcF = m3(kc1, pcmBc_, ec1s);
  cd XcG = cmul(nc, ec2);
  cd XcH = cmul(mk(-1, 0), m3(kc2, nc, ec2s));
  cd Xcz = cmul(Pcj, slopec);
  cd WcB = csub(cmul(pc0mFc_, ec1), m3(kc1, pc0mFc_, ec1s));
  cd WcC = cadd(cmul(mk(-1, 0), cmul(pc0mHc_, ec2)), m3(kc2, pc0mHc_, ec2s));
  cd WcD = cmul(mk(-1, 0), cmul(pc0mFc_, ec1));
  cd WcF = cadd(kc1ec1, m3(kc1, pc0mFc_, ec1s));
  cd WcG = cmul(pc0mHc_, ec2);
  cd WcH = csub(cmul(mk(-1, 0), kc2ec2), m3(kc2, pc0mHc_, ec2s));
  cd Wcz = cmul(Pc0, slopec);
  r = dZ ? dZ[2] : NULL;
  if (r) {
    const cd GmDc = csub(Gc, Dc), GmD = csub(G, D);
    for (int c = 0; c < 22; ++c) r[c] = mk(0, 0);
    r[0] = cmul(fX, XA);
    r[1] = cadd(cmul(fX, XB), cmul(fW, WB));
    r[2] = cadd(cmul(fX, XC), cmul(fW, WC));
    r[3] = csub(cadd(cmul(fX, XD), cmul(fW, WD)), cmul(GmDc, z));
    r[4] = cadd(cmul(fX, XF), cmul(fW, WF));
    r[5] = cadd(cadd(cmul(fX, XG), cmul(fW, WG)), cmul(GmDc, z));
    r[6] = cadd(cmul(fX, XH), cmul(fW, WH));
    r[7] = cmul(fXc, XcA);
    r[8] = cadd(cmul(fXc, XcB), cmul(fWc, WcB));
    r[9] = cadd(cmul(fXc, XcC), cmul(fWc, WcC));
    r[10] = csub(cadd(cmul(fXc, XcD), cmul(fWc, WcD)), cmul(GmD, z));
    r[11] = cadd(cmul(fXc, XcF), cmul(fWc, WcF));
    r[12] = cadd(cadd(cmul(fXc, XcG), cmul(fWc, WcG)), cmul(GmD, z));
    r[13] = cadd(cmul(fXc, XcH), cmul(fWc, WcH));
    r[13 + j] = csub(cmul(W, Xc), cmul(m3(z2, X, Wc), iU2));
    cd t = csub(GD, cmul(X, Xc));
    t = cadd(t, cmul(cmul(mk(2, 0), z), cmul(cmul(X, Wc), iU)));
    t = csub(t, cmul(W, Wc));
    t = cadd(t, cadd(cadd(cmul(fX, Xz), cmul(fW, Wz)), cadd(cmul(fXc, Xcz), cmul(fWc, Wcz))));
    r[21] = t;
  }
  if (dq) {
    cd* g = dq[2];
    g[0] = cmul(fW, cmul(z, slope));      /* P0 through W */
    g[1] = cmul(fX, cmul(z, slope));      /* Pj through X */
    g[2] = cmul(fWc, cmul(z, slopec));    /* Pc0 through Wc */
    g[3] = cmul(fXc, cmul(z, slopec));    /* Pcj through Xc */
    g[4] = cmul(fX, cmul(a, csub(one, k2e2)));     /* Qj through X */
    g[5] = cmul(fXc, cmul(ac, csub(one, kc2ec2))); /* Qcj through Xc */
  }
}

void or_fsys(const double* Z, const double* q, double* out) {
  links L; unpack_links(Z, &L);
  for (int j = 1; j <= 7; ++j) {
    cd f[3];
    eqs_j(&L, ld(Z, 13 + j), j, q, f, NULL, NULL);
    st(out, j - 1, f[0]); st(out, j + 6, f[1]); st(out, j + 13, f[2]);
  }
}

static int row_of(int fam, int j) { return fam == 0 ? j - 1 : (fam == 1 ? j + 6 : j + 13); }

void or_jvar(const double* Z, const double* q, double* out) {
  links L; unpack_links(Z, &L);
  memset(out, 0, sizeof(double) * 2 * 21 * 22);
  for (int j = 1; j <= 7; ++j) {
    cd f[3], dZ[3][22];
    eqs_j(&L, ld(Z, 13 + j), j, q, f, dZ, NULL);
    for (int fam = 0; fam < 3; ++fam)
      for (int c = 0; c < 22; ++c) st(out, row_of(fam, j) * 22 + c, dZ[fam][c]);
  }
}

static int pcol(int k, int j) {
  switch (k) { case 0: return 0; case 1: return j; case 2: return 8; case 3: return 8 + j;
               case 4: return 15 + j; default: return 22 + j; }
}

void or_jpar(const double* Z, const double* q, double* out) {
  links L; unpack_links(Z, &L);
  memset(out, 0, sizeof(double) * 2 * 21 * 30);
  for (int j = 1; j <= 7; ++j) {
    cd f[3], dq[3][6];
    eqs_j(&L, ld(Z, 13 + j), j, q, f, NULL, dq);
    for (int fam = 0; fam < 3; ++fam)
      for (int k = 0; k < 6; ++k) st(out, row_of(fam, j) * 30 + pcol(k, j), dq[fam][k]);
  }
}

/* ------------------------------------------------------------------------- */
/* Homotopy support (htpysupport.cu).                                          */
/* ------------------------------------------------------------------------- */

/* The tracked system: Stephenson II (p NULL; nv 21, np 30) or a generated plug-in.
 * The path state is Y = [Z (nv), Z0, t] (ny = nv + 2 entries), H has nz = nv + 1
 * rows, and the tracker's matrices are ny x ny, row-major with stride ny. */
typedef struct or_plugin or_plugin;
typedef struct { int nv, np; const or_plugin* p; } osys;
static const osys STEPH = {OR_NV, OR_NP, NULL};
#define NY_(S) ((S)->nv + 2)
#define NZ_(S) ((S)->nv + 1)

/* q(t) = (gamma (1-t) spm + t fpm) / (gamma (1-t) + t)   (htpysupport.cu:37-48) */
static void q_s(const osys* S, double t, const double* spm, const double* fpm, const double* gamma, double* out) {
  cd g = mk(gamma[0], gamma[1]);
  cd g1t = cmul(g, mk(1.0 - t, 0));
  cd den = cadd(g1t, mk(t, 0));
  for (int i = 0; i < S->np; ++i)
    st(out, i, cdiv(cadd(cmul(g1t, ld(spm, i)), cmul(mk(t, 0), ld(fpm, i))), den));
}
void or_q(double t, const double* spm, const double* fpm, const double* gamma, double* out) {
  q_s(&STEPH, t, spm, fpm, gamma, out);
}

/* dq/dt = gamma (fpm - spm) / (gamma (1-t) + t)^2   (htpysupport.cu:51-62) */
static void dqdt_s(const osys* S, double t, const double* spm, const double* fpm, const double* gamma,
                   double* out) {
  cd g = mk(gamma[0], gamma[1]);
  cd den = cadd(cmul(g, mk(1.0 - t, 0)), mk(t, 0));
  den = cmul(den, den);
  for (int i = 0; i < S->np; ++i) st(out, i, cdiv(cmul(csub(ld(fpm, i), ld(spm, i)), g), den));
}
void or_dqdt(double t, const double* spm, const double* fpm, const double* gamma, double* out) {
  dqdt_s(&STEPH, t, spm, fpm, gamma, out);
}

static void plugin_rows(const osys* S, const double* Y, const double* q, const double* dq, double* M,
                        double* F);

/* H = [F(Z; q(t)); u . Y - 1]   (htpysupport.cu:64-86) */
static void h_s(const osys* S, const double* Y, const double* u, const double* spm, const double* fpm,
                const double* gamma, double* out) {
  double q[2 * OR_NP];
  const int ny = NY_(S);
  q_s(S, Y[2 * (ny - 1)], spm, fpm, gamma, q);
  if (S->p) {
    double M[2 * OR_NY * OR_NY], dq[2 * OR_NP];
    memset(dq, 0, sizeof(dq));
    plugin_rows(S, Y, q, dq, M, out);
  } else {
    or_fsys(Y, q, out);
  }
  cd d = mk(0, 0);
  for (int i = 0; i < ny; ++i) d = cadd(d, cmul(ld(u, i), ld(Y, i)));
  st(out, S->nv, csub(d, mk(1, 0)));
}
void or_h(const double* Y, const double* u, const double* spm, const double* fpm,
          const double* gamma, double* out) {
  h_s(&STEPH, Y, u, spm, fpm, gamma, out);
}

/* JH = [dF/dZ | dF/dq . dq/dt ; u], nz x ny row-major   (htpysupport.cu:89-144) */
static void jh_s(const osys* S, const double* Y, const double* u, const double* spm, const double* fpm,
                 const double* gamma, double* out) {
  double q[2 * OR_NP], dq[2 * OR_NP];
  const int ny = NY_(S);
  double t = Y[2 * (ny - 1)];
  q_s(S, t, spm, fpm, gamma, q);
  dqdt_s(S, t, spm, fpm, gamma, dq);
  if (S->p) {
    plugin_rows(S, Y, q, dq, out, NULL);
    for (int c = 0; c < ny; ++c) st(out, S->nv * ny + c, ld(u, c));
    return;
  }
  links L; unpack_links(Y, &L);
  for (int j = 1; j <= 7; ++j) {
    cd f[3], dZ[3][22], dP[3][6];
    eqs_j(&L, ld(Y, 13 + j), j, q, f, dZ, dP);
    for (int fam = 0; fam < 3; ++fam) {
      int r = row_of(fam, j);
      for (int c = 0; c < 22; ++c) st(out, r * 23 + c, dZ[fam][c]);
      cd b = mk(0, 0);
      for (int k = 0; k < 6; ++k) b = cadd(b, cmul(dP[fam][k], ld(dq, pcol(k, j))));
      st(out, r * 23 + 22, b);
    }
  }
  for (int c = 0; c < OR_NY; ++c) st(out, 21 * 23 + c, ld(u, c));
}
void or_jh(const double* Y, const double* u, const double* spm, const double* fpm,
           const double* gamma, double* out) {
  jh_s(&STEPH, Y, u, spm, fpm, gamma, out);
}

/* SwitchPatch: rescale Z so that unew . [Z, t] = 1   (htpysupport.cu:9-34) */
static void switch_patch_s(const osys* S, const double* u, const double* Yold, double* Ynew) {
  const int nz = NZ_(S);
  cd den = mk(0, 0);
  for (int i = 0; i < nz; ++i) den = cadd(den, cmul(ld(u, i), ld(Yold, i)));
  cd t = ld(Yold, nz);
  cd s = cdiv(csub(mk(1, 0), cmul(ld(u, nz), t)), den);
  for (int i = 0; i < nz; ++i) st(Ynew, i, cmul(s, ld(Yold, i)));
  st(Ynew, nz, t);
}
void or_switch_patch(const double* u, const double* Yold, double* Ynew) {
  switch_patch_s(&STEPH, u, Yold, Ynew);
}

/* Dense LU with partial pivoting on |a|^2 (first maximum wins), rows swapped by
 * pointer, then back substitution   (htpysupport.cu:146-232). nelim = number of
 * rows that take part (23 for the tangent solve; 22 for Newton, whose last unknown
 * is fixed to xlast, htpysupport.cu:302-400). */
static void lu_solve(int n, cd* mat, cd* b, cd* x, int nelim, int fix_last, cd xlast) {
  cd* a[OR_NY];
  for (int i = 0; i < n; ++i) a[i] = mat + i * n;
  for (int i = 0; i < n; ++i) {
    double maxAbs = 0.0; int maxRow = i;
    for (int k = i; k < nelim; ++k) {
      double v = cnorm2(a[k][i]);
      if (v > maxAbs) { maxAbs = v; maxRow = k; }
    }
    if (maxRow != i) {
      cd* tp = a[i]; a[i] = a[maxRow]; a[maxRow] = tp;
      cd tb = b[i]; b[i] = b[maxRow]; b[maxRow] = tb;
    }
    for (int j = i + 1; j < nelim; ++j) {
      a[j][i] = cdiv(a[j][i], a[i][i]);
      for (int k = i + 1; k < n; ++k) a[j][k] = csub(a[j][k], cmul(a[i][k], a[j][i]));
      b[j] = csub(b[j], cmul(b[i], a[j][i]));
    }
  }
  int top = n - 1;
  if (fix_last) { x[n - 1] = xlast; top = n - 2; }
  for (int i = top; i >= 0; --i) {
    cd sum = mk(0, 0);
    for (int k = i + 1; k < n; ++k) sum = cadd(cmul(a[i][k], x[k]), sum);
    x[i] = cmul(cinv(a[i][i]), csub(b[i], sum));
  }
}

void or_linear_solve(double* mat, double* b, double* x) {
  lu_solve(OR_NY, (cd*)mat, (cd*)b, (cd*)x, OR_NY, 0, mk(0, 0));
}

/* Scale each of the first `rows` rows by 1/max(|re|,|im|) of that row
 * (htpysupport.cu:259-277 and :446-471). */
static void row_scale(int ny, cd* m, int rows, cd* h) {
  for (int i = 0; i < rows; ++i) {
    double mx = 0.0;
    for (int j = 0; j < ny; ++j) {
      if (fabs(m[i * ny + j].re) > mx) mx = fabs(m[i * ny + j].re);
      if (fabs(m[i * ny + j].im) > mx) mx = fabs(m[i * ny + j].im);
    }
    double s = 1.0 / mx;
    if (h) h[i] = cscal(s, h[i]);
    for (int j = 0; j < ny; ++j) m[i * ny + j] = cscal(s, m[i * ny + j]);
  }
}

static double vnorm(const cd* v, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += cnorm2(v[i]);
  return sqrt(s);
}

/* IVP: tangent dY/ds from [JH; Vc] dY = e_23, normalised to unit length with
 * real dt/ds (arclength) or to dt = 1 (t-stepping)   (htpysupport.cu:237-299). */
static void ivp_s(const osys* S, int tstepQ, const double* Yc, const double* Vc, const double* u,
                  const double* spm, const double* fpm, const double* gamma, double* out) {
  const int ny = NY_(S), nz = NZ_(S);
  cd M[OR_NY * OR_NY], b[OR_NY], x[OR_NY];
  jh_s(S, Yc, u, spm, fpm, gamma, (double*)M);
  for (int j = 0; j < ny; ++j) M[nz * ny + j] = ld(Vc, j);
  row_scale(ny, M, nz, NULL);
  for (int i = 0; i < ny; ++i) b[i] = mk(0, 0);
  b[nz] = mk(1, 0);
  lu_solve(ny, M, b, x, ny, 0, mk(0, 0));
  cd sc;
  if (!tstepQ) {
    double th = atan2(x[nz].im, x[nz].re);
    sc = cmul(mk(cos(th), -sin(th)), mk(1.0 / vnorm(x, ny), 0));
  } else {
    sc = cinv(x[nz]);
  }
  for (int i = 0; i < ny; ++i) st(out, i, cmul(sc, x[i]));
  out[2 * nz + 1] = 0.0;
}
void or_ivp(int tstepQ, const double* Yc, const double* Vc, const double* u, const double* spm,
            const double* fpm, const double* gamma, double* out) {
  ivp_s(&STEPH, tstepQ, Yc, Vc, u, spm, fpm, gamma, out);
}

/* Dormand-Prince 6(5), 8 stages; stage i's velocity patch is k_{i-1}
 * (rungekutta.cu:3-123). */
static const double DP_A[8][7] = {
  {0},
  {1. / 10.},
  {-2. / 81., 20. / 81.},
  {615. / 1372., -270. / 343., 1053. / 1372.},
  {3243. / 5500., -54. / 55., 50949. / 71500., 4998. / 17875.},
  {-26492. / 37125., 72. / 55., 2808. / 23375., -24206. / 37125., 338. / 459.},
  {5561. / 2376., -35. / 11., -24117. / 31603., 899983. / 200772., -5225. / 1836., 3925. / 4056.},
  {465467. / 266112., -2945. / 1232., -5610201. / 14158144., 10513573. / 3212352., -424325. / 205632.,
   376225. / 454272.}};
static const double DP_E[8] = {-13. / 2400., 0., 19683. / 618800., -2401. / 31200., 65. / 816.,
                               -15. / 416., -521. / 5600., 1. / 10.};
static const double DP_B[8] = {61. / 864., 0., 98415. / 321776., 16807. / 146016., 1375. / 7344.,
                               1375. / 5408., -37. / 1120., 1. / 10.};

/* sum_{i<n} w[i] s k[i], accumulated from the last term to the first as the
 * reference's nested .add() chains do. */
static void comb(int ny, double s, const double* w, cd k[8][OR_NY], int n, cd* out) {
  for (int e = 0; e < ny; ++e) {
    cd acc = mk(0, 0);
    int first = 1;
    for (int i = n - 1; i >= 0; --i) {
      if (w[i] == 0.0) continue;
      cd term = cscal(w[i] * s, k[i][e]);
      acc = first ? term : cadd(term, acc);
      first = 0;
    }
    out[e] = acc;
  }
}

static void dp65_s(const osys* S, double s, double tol, int tstepQ, const double* Yc, const double* Vc,
                   const double* u, const double* spm, const double* fpm, const double* gamma, double* Yn,
                   double* Vn, double* err, double* scale) {
  const int ny = NY_(S);
  cd k[8][OR_NY];
  cd Yarg[OR_NY], d[OR_NY];
  ivp_s(S, tstepQ, Yc, Vc, u, spm, fpm, gamma, (double*)k[0]);
  for (int stg = 1; stg < 8; ++stg) {
    comb(ny, s, DP_A[stg], k, stg, d);
    for (int e = 0; e < ny; ++e) Yarg[e] = cadd(ld(Yc, e), d[e]);
    ivp_s(S, tstepQ, (double*)Yarg, (double*)k[stg - 1], u, spm, fpm, gamma, (double*)k[stg]);
  }
  comb(ny, s, DP_E, k, 8, d);
  *err = vnorm(d, ny);
  if (*err > 10e-17) *scale = 0.8 * pow(tol / (*err), 1. / 6.);
  else *scale = 5.0;
  if (*scale > 5) *scale = 5;
  comb(ny, s, DP_B, k, 8, d);
  for (int e = 0; e < ny; ++e) st(Yn, e, cadd(ld(Yc, e), d[e]));
  memcpy(Vn, k[7], sizeof(cd) * ny);
}
void or_dp65(double s, double tol, int tstepQ, const double* Yc, const double* Vc, const double* u,
             const double* spm, const double* fpm, const double* gamma, double* Yn, double* Vn,
             double* err, double* scale) {
  dp65_s(&STEPH, s, tol, tstepQ, Yc, Vc, u, spm, fpm, gamma, Yn, Vn, err, scale);
}

/* Newton corrector with t fixed at tgoal, row-scaled J and H   (htpysupport.cu:407-494) */
static int newton_impl(const osys* S, double tgoal, const double* Vn, const double* u, const double* spm,
                       const double* fpm, const double* gamma, int maxIts, double tol,
                       int residualtype, double* YN, double* residual) {
  const int ny = NY_(S), nz = NZ_(S);
  int i = 0;
  *residual = 100.0;
  while (i < maxIts && *residual > tol) {
    cd M[OR_NY * OR_NY], h[OR_NY], bb[OR_NY], dY[OR_NY];
    jh_s(S, YN, u, spm, fpm, gamma, (double*)M);
    for (int j = 0; j < ny; ++j) M[nz * ny + j] = ld(Vn, j);
    h_s(S, YN, u, spm, fpm, gamma, (double*)h);
    row_scale(ny, M, nz, h);
    double tdiff = tgoal - YN[2 * nz];
    for (int j = 0; j < nz; ++j) bb[j] = cscal(-1.0, h[j]);
    bb[nz] = mk(0, 0);
    lu_solve(ny, M, bb, dY, nz, 1, mk(tdiff, 0));
    for (int e = 0; e < ny; ++e) st(YN, e, cadd(ld(YN, e), dY[e]));
    if (residualtype == 0) {
      h_s(S, YN, u, spm, fpm, gamma, (double*)h);
      *residual = vnorm(h, nz);
    } else {
      *residual = vnorm(dY, ny);
    }
    i++;
  }
  return i;
}

void or_newton(double tgoal, const double* Vn, const double* u, const double* spm, const double* fpm,
               const double* gamma, int maxIts, double tol, int residualtype, double* YN,
               double* residual) {
  newton_impl(&STEPH, tgoal, Vn, u, spm, fpm, gamma, maxIts, tol, residualtype, YN, residual);
}

/* Raw Philox block and uniform draw, exported for the known-answer tests. */
void or_philox_block(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  frg_philox4x32_10(ctr, key, out);
}
double or_uniform01(uint64_t seed, uint64_t stream, uint64_t index) {
  return frg_uniform01(seed, stream, index);
}

/* ------------------------------------------------------------------------- */
/* Random draws.                                                               */
/* ------------------------------------------------------------------------- */

typedef struct { uint64_t seed, stream, index; } rng_t;
static inline double urand(rng_t* r) { return frg_uniform01(r->seed, r->stream, r->index++); }
/* One start value: U(-R,R) (frgkinematics.cu:41) or, for start_dist 1, a normal
 * N(0, 1/2) component of a standard complex normal by Box-Muller on two draws. */
static inline double start_draw(const or_config* c, rng_t* r) {
  if (c->start_dist == 0) return 2.0 * c->start_range * urand(r) - c->start_range;
  double u1 = urand(r), u2 = urand(r);
  return sqrt(-log(u1)) * cos(6.283185307179586 * u2);
}

/* GenerateStart: random mechanism -> exact start root and start parameters
 * (frgkinematics.cu:13-136). */
void or_generate_start(const or_config* c, uint64_t seed, uint64_t stream, double* spt, double* spm) {
  rng_t r = {seed, stream, 0};
  cd z[21], P[8], Pc[8], Q[8], Qc[8], RUc[8];
  for (int i = 0; i < 14; ++i) { double re = start_draw(c, &r); double im = start_draw(c, &r); z[i] = mk(re, im); }
  { double re = start_draw(c, &r), im = start_draw(c, &r); P[0] = mk(re, im); }
  { double re = start_draw(c, &r), im = start_draw(c, &r); Pc[0] = mk(re, im); }
  for (int j = 1; j <= 7; ++j) { double re = start_draw(c, &r), im = start_draw(c, &r); RUc[j] = mk(re, im); }
  const cd A = z[0], B = z[1], C = z[2], D = z[3], F = z[4], G = z[5], H = z[6];
  const cd Ac = z[7], Bc = z[8], Cc = z[9], Dc = z[10], Fc = z[11], Gc = z[12], Hc = z[13];
  const cd one = mk(1, 0);
  for (int j = 1; j <= 7; ++j) {
    cd R = RUc[j], iR = cinv(R);
    /* quadratic for T = TUc (frgkinematics.cu:63-80) */
    cd Aq = cmul(csub(G, D), csub(cmul(iR, csub(Hc, Gc)), csub(Hc, Fc)));
    cd Acq = cmul(csub(Gc, Dc), csub(cmul(R, csub(H, G)), csub(H, F)));
    cd Bq = cadd(csub(csub(mk(0, 0), cmul(R, cmul(csub(H, G), csub(Hc, Fc)))),
                      cmul(iR, cmul(csub(Hc, Gc), csub(H, F)))),
                 cadd(cmul(csub(G, D), csub(Gc, Dc)),
                      cadd(cmul(csub(H, G), csub(Hc, Gc)),
                           csub(cmul(csub(H, F), csub(Hc, Fc)), cmul(csub(F, D), csub(Fc, Dc))))));
    double pm = 1.0; if (urand(&r) < 0.5) pm = -1.0;
    cd disc = csqrt_ref(csub(cmul(Bq, Bq), cmul(mk(4, 0), cmul(Aq, Acq))));
    cd TUc = cmul(cinv(cmul(mk(2, 0), Aq)), cadd(csub(mk(0, 0), Bq), cscal(pm, disc)));
    cd SUc = cmul(cinv(csub(F, D)), cadd(cmul(TUc, csub(G, D)), csub(cmul(R, csub(H, G)), csub(H, F))));
    /* quadratic for U_j (frgkinematics.cu:87-107) */
    cd w = csub(csub(cmul(R, csub(H, C)), cmul(SUc, csub(F, B))), csub(H, F));
    cd wc = csub(csub(cmul(iR, csub(Hc, Cc)), cmul(cinv(SUc), csub(Fc, Bc))), csub(Hc, Fc));
    Aq = cmul(csub(Ac, Bc), w);
    Acq = cmul(csub(A, B), wc);
    Bq = cadd(cmul(w, wc), csub(cmul(csub(A, B), csub(Ac, Bc)), cmul(csub(C, A), csub(Cc, Ac))));
    pm = 1.0; if (urand(&r) < 0.5) pm = -1.0;
    disc = csqrt_ref(csub(cmul(Bq, Bq), cmul(mk(4, 0), cmul(Aq, Acq))));
    cd Uj = cmul(cinv(cmul(mk(2, 0), Aq)), cadd(csub(mk(0, 0), Bq), cscal(pm, disc)));
    z[13 + j] = Uj;
    /* prescribed rotations and precision points (frgkinematics.cu:109-120) */
    cd QUc = cmul(cdiv(mk(-1, 0), csub(C, A)), cadd(cmul(cinv(Uj), csub(A, B)), w));
    Q[j] = cmul(QUc, Uj);
    Qc[j] = cinv(Q[j]);
    cd S = cmul(SUc, Uj);
    P[j] = cadd(B, cadd(cmul(S, csub(F, B)), cmul(Uj, csub(P[0], F))));
    Pc[j] = cadd(Bc, cadd(cmul(cinv(S), csub(Fc, Bc)), cmul(cinv(Uj), csub(Pc[0], Fc))));
    (void)one;
  }
  for (int i = 0; i < 21; ++i) st(spt, i, z[i]);
  for (int j = 0; j < 8; ++j) { st(spm, j, P[j]); st(spm, 8 + j, Pc[j]); }
  for (int j = 1; j <= 7; ++j) { st(spm, 15 + j, Q[j]); st(spm, 22 + j, Qc[j]); }
}

/* ------------------------------------------------------------------------- */
/* The path tracker (htpytrack.cu:33-220).                                     */
/* ------------------------------------------------------------------------- */

static void draw_patch(int ny, const or_config* c, rng_t* r, double* u) {
  double R = c->patch_range;
  for (int i = 0; i < ny; ++i) {
    u[2 * i] = 2.0 * R * urand(r) - R;
    u[2 * i + 1] = 2.0 * R * urand(r) - R;
  }
}

static void track_path_s(const osys* sys, const or_config* c, const double* spt, const double* spm,
                         const double* fpm, const double* gamma, uint64_t seed, uint64_t stream,
                         double* Yfinal, int* code, or_stats* stt) {
  const int nv = sys->nv, ny = NY_(sys), it = ny - 1; /* it: index of t in the path state */
  rng_t rng = {seed, stream, 0};  /* the reference hands TrackPath a fresh copy of the state */
  double Vc[2 * OR_NY], Yn[2 * OR_NY], Vn[2 * OR_NY], YN[2 * OR_NY], u[2 * OR_NY];
  double* Yc = Yfinal;            /* htpytrack.cu:46: the working point lives in Yfinal */
  or_stats local; memset(&local, 0, sizeof(local));
  or_stats* S = stt ? stt : &local;
  const size_t ybytes = sizeof(double) * 2 * ny;
  memmove(Yc, spt, sizeof(double) * 2 * nv);
  Yc[2 * nv] = 1.0; Yc[2 * nv + 1] = 0.0;
  Yc[2 * it] = 0.0; Yc[2 * it + 1] = 0.0;
  draw_patch(ny, c, &rng, u);
  switch_patch_s(sys, u, Yc, Yc);
  draw_patch(ny, c, &rng, Vc);
  ivp_s(sys, 0, Yc, Vc, u, spm, fpm, gamma, Vc);
  S->ivp_solves++;

  double s = c->s_init, err = 0, scale = 0, residual = 100.0;
  int tstepQ = 0, streak = c->caution_steps - 1, step = 0, ministep = 0;
  *code = 0;

  for (;;) { /* main loop */
    if (step == c->max_steps) { *code = 1; return; }
    for (;;) { /* correction loop */
      for (;;) { /* final steps loop */
        for (;;) { /* predictor loop */
          dp65_s(sys, s, c->rk_tol, tstepQ, Yc, Vc, u, spm, fpm, gamma, Yn, Vn, &err, &scale);
          S->rk_attempts++; S->ivp_solves += 8;
          if (ministep++ == c->max_ministeps) { *code = 2; return; }
          if (err <= c->rk_tol) break;
          if (s <= c->s_min) { *code = 3; return; }
          s *= scale;
          if (s < c->s_min) s = c->s_min * 0.9;
          streak = 0;
        }
        if (Yn[2 * it] <= 1. - c->nudge_trigger) break;
        if (fabs(1. - Yn[2 * it]) < c->sharp_trigger) break;
        tstepQ = 1;
        s = 1 - Yc[2 * it];
      }
      if (fabs(1. - Yn[2 * it]) < c->sharp_trigger) break;
      int i = 0;
      while (i < c->newt_attempts) {
        memcpy(YN, Yn, ybytes);
        S->newton_iters += newton_impl(sys, Yn[2 * it], Vn, u, spm, fpm, gamma, c->newt_its, c->newt_tol,
                                       c->newt_residual, YN, &residual);
        S->newton_calls++;
        if (ministep++ == c->max_ministeps) { *code = 2; return; }
        if (residual < c->newt_tol) break;
        draw_patch(ny, c, &rng, u);
        switch_patch_s(sys, u, Yn, Yn);
        i++;
      }
      if (residual < c->newt_tol) break;
      if (s <= c->s_min) { *code = 4; return; }
      s *= 0.5;
      if (s < c->s_min) s = c->s_min * 0.9;
      streak = 0;
    }
    if (fabs(1. - Yn[2 * it]) < c->sharp_trigger) break;
    memcpy(Yc, YN, ybytes);
    memcpy(Vc, Vn, ybytes);
    streak++;
    if (streak < c->caution_steps && scale > 1.) scale = 1.;
    s *= scale;
    if (s > c->s_max) s = c->s_max;
    else if (s < c->s_min) s = c->s_min * 0.9;
    step++;
    S->steps++;
  }
  /* sharpening at t = 1 (htpytrack.cu:194-216) */
  int i = 0;
  while (i < c->sharp_attempts) {
    memcpy(Yfinal, Yn, ybytes);
    S->newton_iters += newton_impl(sys, 1., Vn, u, spm, fpm, gamma, c->sharp_its, c->sharp_tol,
                                   c->sharp_residual, Yfinal, &residual);
    S->newton_calls++;
    if (ministep++ == c->max_ministeps) { *code = 2; return; }
    if (residual < c->sharp_tol) break;
    draw_patch(ny, c, &rng, u);
    switch_patch_s(sys, u, Yn, Yn);
    i++;
  }
  if (residual >= c->sharp_tol) *code = 5;
}

void or_track_path(const or_config* c, const double* spt, const double* spm, const double* fpm,
                   const double* gamma, uint64_t seed, uint64_t stream, double* Yfinal, int* code,
                   or_stats* stt) {
  track_path_s(&STEPH, c, spt, spm, fpm, gamma, seed, stream, Yfinal, code, stt);
}

/* ------------------------------------------------------------------------- */
/* Plug-in systems: the generated rows and starts of the modules in            */
/* finite_root_generation_gb300/systems (frg_plugins_gen.h).                   */
/* ------------------------------------------------------------------------- */

/* A x = b (n x n, row-major; A and b overwritten): Gaussian elimination with partial
 * pivoting on |a|^2, the first maximum winning, for the start parameters. */
static void small_solve(int n, cd* A, cd* b, cd* x) {
  for (int i = 0; i < n; ++i) {
    int br = i;
    double best = cnorm2(A[i * n + i]);
    for (int k = i + 1; k < n; ++k) {
      double v = cnorm2(A[k * n + i]);
      if (v > best) { best = v; br = k; }
    }
    if (br != i) {
      for (int c = 0; c < n; ++c) { cd t = A[i * n + c]; A[i * n + c] = A[br * n + c]; A[br * n + c] = t; }
      cd t = b[i]; b[i] = b[br]; b[br] = t;
    }
    for (int j = i + 1; j < n; ++j) {
      cd l = cdiv(A[j * n + i], A[i * n + i]);
      for (int c = i + 1; c < n; ++c) A[j * n + c] = csub(A[j * n + c], cmul(l, A[i * n + c]));
      b[j] = csub(b[j], cmul(l, b[i]));
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    cd sum = b[i];
    for (int c = i + 1; c < n; ++c) sum = csub(sum, cmul(A[i * n + c], x[c]));
    x[i] = cdiv(sum, A[i * n + i]);
  }
}

struct or_plugin {
  int id;
  const char* name;
  int nv, np;
  /* rows 0..nv-1 of JH into M (stride ld): dF/dZ, dF/dZ0, the t column; F if given */
  void (*rows)(const cd* Y, const cd* q, const cd* dq, cd* M, int ld, cd* F);
  /* start root z and start parameters q from the random stream r */
  void (*start)(const or_config* c, rng_t* r, cd* z, cd* q);
};

#include "frg_plugins_gen.h"

static void plugin_rows(const osys* S, const double* Y, const double* q, const double* dq, double* M,
                        double* F) {
  S->p->rows((const cd*)Y, (const cd*)q, (const cd*)dq, (cd*)M, NY_(S), (cd*)F);
}

static int plugin_sys(int system, osys* out) {
  for (int k = 0; k < OR_NUM_PLUGINS; ++k)
    if (OR_PLUGINS[k].id == system) {
      out->nv = OR_PLUGINS[k].nv;
      out->np = OR_PLUGINS[k].np;
      out->p = &OR_PLUGINS[k];
      return 1;
    }
  return 0;
}

int or_num_plugins(void) { return OR_NUM_PLUGINS; }

int or_plugin_info(int system, int* nv, int* np) {
  osys S;
  if (!plugin_sys(system, &S)) return 0;
  *nv = S.nv;
  *np = S.np;
  return 1;
}

int or_plugin_rows(int system, const double* Y, const double* q, const double* dq, double* M, double* F) {
  osys S;
  if (!plugin_sys(system, &S)) return 0;
  plugin_rows(&S, Y, q, dq, M, F);
  return 1;
}

int or_plugin_start(int system, const or_config* c, uint64_t seed, uint64_t stream, double* spt, double* spm) {
  osys S;
  if (!plugin_sys(system, &S)) return 0;
  rng_t r = {seed, stream, 0};
  S.p->start(c, &r, (cd*)spt, (cd*)spm);
  return 1;
}

/* One plug-in path: start, track, dehomogenize (the root as tracked), and the
 * row-scaled residual max_i |F_i| / max_c |dF_i/dZ_c| of the target system at the root. */
static void plugin_path(const osys* S, const or_config* c, uint64_t seed, uint64_t stream, const double* fpm,
                        const double* gamma, double* root, int* code, double* Yfinal, double* resid) {
  const int nv = S->nv, ny = NY_(S), nz = NZ_(S);
  double spt[2 * OR_NV], spm[2 * OR_NP], Y[2 * OR_NY], u[2 * OR_NY];
  rng_t r = {seed, stream, 0};
  S->p->start(c, &r, (cd*)spt, (cd*)spm);
  track_path_s(S, c, spt, spm, fpm, gamma, seed, stream, Y, code, NULL);
  if (Yfinal) memcpy(Yfinal, Y, sizeof(double) * 2 * ny);
  memset(u, 0, sizeof(u));
  u[2 * nv] = 1.0;
  switch_patch_s(S, u, Y, Y);
  memcpy(root, Y, sizeof(double) * 2 * nv);
  if (resid) {
    double Yr[2 * OR_NY], dq[2 * OR_NP], M[2 * OR_NY * OR_NY], F[2 * OR_NY];
    memcpy(Yr, Y, sizeof(double) * 2 * nv);
    Yr[2 * nv] = 1.0; Yr[2 * nv + 1] = 0.0;
    Yr[2 * (nv + 1)] = 1.0; Yr[2 * (nv + 1) + 1] = 0.0;
    memset(dq, 0, sizeof(dq));
    plugin_rows(S, Yr, fpm, dq, M, F);
    double rmax = 0.0;
    for (int i = 0; i < nv; ++i) {
      double mx = 0.0;
      for (int e = 0; e < nz; ++e) {
        mx = fmax(mx, fabs(M[2 * (i * ny + e)]));
        mx = fmax(mx, fabs(M[2 * (i * ny + e) + 1]));
      }
      double ri = sqrt(F[2 * i] * F[2 * i] + F[2 * i + 1] * F[2 * i + 1]) / mx;
      rmax = (ri == ri) ? fmax(rmax, ri) : INFINITY;
    }
    *resid = rmax;
  }
}

typedef struct {
  const osys* S; const or_config* c; uint64_t seed; const uint64_t* streams; int64_t n; int ntasks;
  const int64_t* task_start; const double* fpm; const double* gamma; double* roots; int* codes;
  double* yfinal; double* resid; int nthreads; int w;
} plugin_arg;

static void* plugin_worker(void* p) {
  plugin_arg* a = (plugin_arg*)p;
  const int nv = a->S->nv, ny = NY_(a->S), np = a->S->np;
  for (int64_t i = a->w; i < a->n; i += a->nthreads) {
    int k = 0;
    while (k + 1 < a->ntasks && a->task_start[k + 1] <= i) ++k;
    plugin_path(a->S, a->c, a->seed, a->streams[i], a->fpm + 2 * np * k, a->gamma + 2 * k, a->roots + 2 * nv * i,
                a->codes + i, a->yfinal ? a->yfinal + 2 * ny * i : NULL, a->resid ? a->resid + i : NULL);
  }
  return NULL;
}

int or_plugin_batch(int system, const or_config* c, uint64_t seed, const uint64_t* streams, int64_t n, int ntasks,
                    const int64_t* task_start, const double* fpm, const double* gamma, double* roots, int* codes,
                    double* yfinal, double* resid, int nthreads) {
  osys S;
  if (!plugin_sys(system, &S)) return 0;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  plugin_arg args[256];
  for (int w = 0; w < nthreads; ++w) {
    plugin_arg a = {&S, c, seed, streams, n, ntasks, task_start, fpm, gamma, roots, codes, yfinal, resid,
                    nthreads, w};
    args[w] = a;
    pthread_create(&th[w], NULL, plugin_worker, &args[w]);
  }
  for (int w = 0; w < nthreads; ++w) pthread_join(th[w], NULL);
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Cognates (frgkinematics.cu:185-285).                                        */
/* ------------------------------------------------------------------------- */

/* Cognate12: the 1/2 cognate of one side (A..H or Ac..Hc)   (frgkinematics.cu:185-224). */
static void cognate12(const cd* o, cd P, cd* out) {
  cd A = o[0], B = o[1], C = o[2], D = o[3], F = o[4], G = o[5], H = o[6];
  cd sc = cdiv(csub(B, F), csub(D, F));
  cd Dp = cadd(cmul(sc, csub(D, H)), H);
  cd Gp = cadd(cmul(sc, csub(G, H)), H);
  sc = cdiv(csub(P, F), csub(H, F));
  out[0] = cadd(cmul(sc, csub(A, B)), B);
  out[1] = B;
  out[2] = cadd(cmul(sc, csub(C, B)), B);
  out[3] = cadd(cmul(sc, csub(Dp, B)), B);
  out[4] = cadd(B, csub(P, F));
  out[5] = cadd(cmul(sc, csub(Gp, B)), B);
  out[6] = cadd(cmul(sc, csub(H, B)), B);
}

/* CognateSolns: the root and its 1/2 cognate, the one with the smaller Re(A) first
 * (frgkinematics.cu:227-285). */
void or_cognate(const double* z, const double* q, double* out) {
  cd r0[21], r1[21];
  for (int i = 0; i < 21; ++i) r0[i] = ld(z, i);
  cd B = r0[1], F = r0[4], P0 = ld(q, 0), Pc0 = ld(q, 8);
  for (int i = 1; i <= 7; ++i)
    r1[13 + i] = cdiv(csub(csub(ld(q, i), B), cmul(r0[13 + i], csub(P0, F))), csub(F, B));
  cognate12(r0, P0, r1);
  cognate12(r0 + 7, Pc0, r1 + 7);
  int swap = r1[0].re < r0[0].re;
  for (int i = 0; i < 21; ++i) {
    st(out, i, swap ? r1[i] : r0[i]);
    st(out, 21 + i, swap ? r0[i] : r1[i]);
  }
}

/* The reference kernel body for one path (frg.cu:41-68). Yfinal, if given,
 * receives the tracked point before dehomogenizing. */
void or_homotopy_path(const or_config* c, uint64_t seed, uint64_t stream, const double* fpm,
                      const double* gamma, double* root, int* code, double* Yfinal, or_stats* st_) {
  double spt[2 * 21], spm[2 * OR_NP], Y[2 * OR_NY], u[2 * OR_NY];
  or_generate_start(c, seed, stream, spt, spm);
  or_track_path(c, spt, spm, fpm, gamma, seed, stream, Y, code, st_);
  if (Yfinal) memcpy(Yfinal, Y, sizeof(Y));
  memset(u, 0, sizeof(u));
  u[2 * 21] = 1.0;
  or_switch_patch(u, Y, Y);
  double cog[2 * 42];
  or_cognate(Y, fpm, cog);
  memcpy(root, cog, sizeof(double) * 42);
}

typedef struct {
  const or_config* c; uint64_t seed; const uint64_t* streams; int64_t n; const double* fpm;
  const double* gamma; double* roots; int* codes; double* yfinal; int64_t* work; int nthreads; int w;
} batch_arg;

static void* batch_worker(void* p) {
  batch_arg* a = (batch_arg*)p;
  for (int64_t i = a->w; i < a->n; i += a->nthreads) {
    or_stats s; memset(&s, 0, sizeof(s));
    or_homotopy_path(a->c, a->seed, a->streams[i], a->fpm, a->gamma, a->roots + 42 * i, a->codes + i,
                     a->yfinal ? a->yfinal + 2 * OR_NY * i : NULL, &s);
    if (a->work) { a->work[3 * i] = s.ivp_solves; a->work[3 * i + 1] = s.newton_iters; a->work[3 * i + 2] = s.steps; }
  }
  return NULL;
}

void or_homotopy_batch(const or_config* c, uint64_t seed, const uint64_t* streams, int64_t n,
                       const double* fpm, const double* gamma, double* roots, int* codes,
                       double* yfinal, int64_t* work, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  pthread_t th[256];
  batch_arg args[256];
  if (nthreads > 256) nthreads = 256;
  for (int w = 0; w < nthreads; ++w) {
    batch_arg a = {c, seed, streams, n, fpm, gamma, roots, codes, yfinal, work, nthreads, w};
    args[w] = a;
    pthread_create(&th[w], NULL, batch_worker, &args[w]);
  }
  for (int w = 0; w < nthreads; ++w) pthread_join(th[w], NULL);
}

/* ------------------------------------------------------------------------- */
/* Collection merge with duplicate marking (frgsupport.cu:10-215).            */
/* ------------------------------------------------------------------------- */

typedef struct { double key; int64_t idx; } keyidx;
static int cmp_keyidx(const void* x, const void* y) {
  const keyidx* a = (const keyidx*)x; const keyidx* b = (const keyidx*)y;
  if (a->key < b->key) return -1;
  if (a->key > b->key) return 1;
  return (a->idx > b->idx) - (a->idx < b->idx);
}

static int same_root(const double* a, const double* b, double tol) {
  for (int j = 0; j < 42; ++j)
    if (fabs(a[j] - b[j]) > tol) return 0;
  return 1;
}

/* Merge the new roots into the sorted collection: new roots are ordered by Re(root[0])
 * with ties in index order (the stable sort of frg.cu:432-435); a new root goes before
 * a collected root only when strictly smaller (frgsupport.cu:37). A successful new root
 * is a duplicate (code 6) when all 42 reals are within tol of a collected root, or of
 * a lower-index new root that is still a success, among its neighbours within tol in
 * Re(root[0]) (frgsupport.cu:69-172). Non-duplicate successes are folded into the
 * collection (frgsupport.cu:191-211). Returns the new collection size. */
int64_t or_sort_merge(const double* coll, int64_t ncoll, const double* fpt, int* codes, int64_t n,
                      double tol, double* coll_out) {
  keyidx* ord = (keyidx*)malloc(sizeof(keyidx) * (size_t)(n > 0 ? n : 1));
  for (int64_t i = 0; i < n; ++i) { ord[i].key = fpt[42 * i]; ord[i].idx = i; }
  qsort(ord, (size_t)n, sizeof(keyidx), cmp_keyidx);
  int64_t total = ncoll + n;
  /* merged order: entries >= 0 are collection indices, < 0 are -(new index) - 1 */
  int64_t* merged = (int64_t*)malloc(sizeof(int64_t) * (size_t)(total > 0 ? total : 1));
  int64_t* rank_of_new = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int64_t ic = 0, in = 0, m = 0;
  while (ic < ncoll || in < n) {
    if (in < n && (ic >= ncoll || fpt[42 * ord[in].idx] < coll[42 * ic])) {
      rank_of_new[ord[in].idx] = m; merged[m++] = -ord[in].idx - 1; in++;
    } else {
      merged[m++] = ic++;
    }
  }
  for (int64_t t = 0; t < n; ++t) {
    if (codes[t] != 0) continue;
    const double* rt = fpt + 42 * t;
    int64_t r = rank_of_new[t];
    for (int dir = -1; dir <= 1; dir += 2) {
      for (int64_t k = r + dir; k >= 0 && k < total; k += dir) {
        int64_t e = merged[k];
        const double* ro = e >= 0 ? coll + 42 * e : fpt + 42 * (-e - 1);
        if (fabs(rt[0] - ro[0]) > tol) break;
        if (e >= 0) {
          if (same_root(rt, ro, tol)) codes[t] = 6;
        } else {
          int64_t u = -e - 1;
          if (u < t && codes[u] == 0 && same_root(rt, ro, tol)) codes[t] = 6;
        }
      }
    }
  }
  int64_t out = 0;
  for (int64_t k = 0; k < total; ++k) {
    int64_t e = merged[k];
    if (e >= 0) memcpy(coll_out + 42 * out++, coll + 42 * e, sizeof(double) * 42);
    else if (codes[-e - 1] == 0) memcpy(coll_out + 42 * out++, fpt + 42 * (-e - 1), sizeof(double) * 42);
  }
  free(ord); free(merged); free(rank_of_new);
  return out;
}

/* Principal branch W0 of the Lambert W function by Halley's iteration on w e^w = z,
 * used for the coverage estimate s W(-e^{-1/s}/s) + 1 (frg.cu:463-464,
 * frgsupport.cu:249-272). Start: the branch-point series near -1/e, log asymptotics
 * for large z, z itself otherwise. */
double or_lambertw0(double z) {
  const double em1 = 0.36787944117144233;
  if (z == 0.0) return 0.0;
  if (z < -em1) return NAN;
  double w;
  if (z < -0.25) {
    double p = sqrt(2.0 * (2.718281828459045 * z + 1.0));
    w = -1.0 + p - p * p / 3.0 + 11.0 / 72.0 * p * p * p;
  } else if (z < 3.0) {
    w = log1p(z) * 0.7;
  } else {
    double l1 = log(z), l2 = log(l1);
    w = l1 - l2 + l2 / l1;
  }
  for (int it = 0; it < 64; ++it) {
    double ew = exp(w), f = w * ew - z;
    double wp1 = w + 1.0;
    double denom = ew * wp1 - (w + 2.0) * f / (2.0 * wp1);
    if (denom == 0.0) break;
    double dw = f / denom;
    w -= dw;
    if (fabs(dw) <= 1e-16 * (1.0 + fabs(w))) break;
  }
  return w;
}
