/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * Plain-C restatement of the reference path tracker (mplecnik/Finite_Root_Generation),
 * used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
 * checker. Each function cites the reference file:line whose algorithm it
 * restates. Complex arrays are interleaved (re, im) doubles in the reference's
 * orders: unknowns Z = [A,B,C,D,F,G,H, Ac..Hc, U1..U7, Z0] (htpykinematics.cu:10-27),
 * path state Y = [Z, t], parameters q = [P0..P7, Pc0..Pc7, Q1..Q7, Qc1..Qc7]
 * (htpykinematics.cu:29-33).
 *
 * Parity pin: the restatement is checked against golden vectors recorded from the
 * reference's own sources compiled for the host (oracle/ref_driver.cpp,
 * tests/golden/make_golden.py) in tests/test_oracle_golden.py.
 */
#ifndef FRG_ORACLE_H
#define FRG_ORACLE_H

#include <stdint.h>

#define OR_NV 21
#define OR_NP 30
#define OR_NY 23

/* Tracker settings; defaults are the reference's compile-time constants. */
typedef struct {
  double s_init, s_max, s_min, rk_tol;        /* htpytrack.cu:9-12 */
  int caution_steps;                          /* htpytrack.cu:13 */
  int newt_its; double newt_tol; int newt_residual; int newt_attempts;   /* :16-19 */
  int sharp_its; double sharp_tol; int sharp_residual; int sharp_attempts; /* :20-23 */
  double sharp_trigger, nudge_trigger;        /* :24-25 */
  int max_steps, max_ministeps;               /* :26-27 */
  double patch_range;                         /* :30-31 (patches U(-2,2)^2) */
  int start_dist;                             /* 0: U(-r,r)^2 (frgkinematics.cu:7-8), 1: complex normal */
  double start_range;                         /* 5 */
} or_config;

typedef struct {
  int64_t rk_attempts;   /* DormandPrince65 calls (8 linear solves each) */
  int64_t ivp_solves;    /* 23x23 tangent solves, including the initial one */
  int64_t newton_iters;  /* 22x22 Newton solves (corrector + sharpening) */
  int64_t steps;         /* accepted steps */
  int64_t newton_calls;
} or_stats;

void or_config_default(or_config* c);

void or_fsys(const double* Z, const double* q, double* out);              /* 21 */
void or_jvar(const double* Z, const double* q, double* out);              /* 21 x 22 */
void or_jpar(const double* Z, const double* q, double* out);              /* 21 x 30 */
void or_q(double t, const double* spm, const double* fpm, const double* gamma, double* out);
void or_dqdt(double t, const double* spm, const double* fpm, const double* gamma, double* out);
void or_h(const double* Y, const double* u, const double* spm, const double* fpm,
          const double* gamma, double* out);                              /* 22 */
void or_jh(const double* Y, const double* u, const double* spm, const double* fpm,
           const double* gamma, double* out);                             /* 22 x 23 */
void or_switch_patch(const double* u, const double* Yold, double* Ynew);
void or_linear_solve(double* mat, double* b, double* x);                  /* 23 x 23, in place */
void or_ivp(int tstepQ, const double* Yc, const double* Vc, const double* u, const double* spm,
            const double* fpm, const double* gamma, double* out);
void or_dp65(double s, double tol, int tstepQ, const double* Yc, const double* Vc, const double* u,
             const double* spm, const double* fpm, const double* gamma, double* Yn, double* Vn,
             double* err, double* scale);
void or_newton(double tgoal, const double* Vn, const double* u, const double* spm, const double* fpm,
               const double* gamma, int maxIts, double tol, int residualtype, double* YN,
               double* residual);
void or_generate_start(const or_config* c, uint64_t seed, uint64_t stream, double* spt, double* spm);
void or_track_path(const or_config* c, const double* spt, const double* spm, const double* fpm,
                   const double* gamma, uint64_t seed, uint64_t stream, double* Yfinal, int* code,
                   or_stats* st);
void or_cognate(const double* z, const double* q, double* out);           /* 2 x 21 */
void or_homotopy_path(const or_config* c, uint64_t seed, uint64_t stream, const double* fpm,
                      const double* gamma, double* root, int* code, double* Yfinal, or_stats* st);
void or_homotopy_batch(const or_config* c, uint64_t seed, const uint64_t* streams, int64_t n,
                       const double* fpm, const double* gamma, double* roots, int* codes,
                       double* yfinal, int64_t* work, int nthreads);
int64_t or_sort_merge(const double* coll, int64_t ncoll, const double* fpt, int* codes, int64_t n,
                      double tol, double* coll_out);
double or_lambertw0(double z);

/* Plug-in systems (finite_root_generation_gb300/systems; system ids 1..): the same
 * tracker on the generated rows and starts. Each returns 0 for an unknown system.
 *   or_plugin_rows   M: nv x (nv + 2) rows of JH, row-major (dF/dZ, dF/dZ0, t column);
 *                    F: nv values (optional)
 *   or_plugin_batch  paths i = 0..n-1 with random streams streams[i]; path i belongs to the
 *                    task k with task_start[k] <= i < task_start[k + 1] (ntasks + 1 entries);
 *                    fpm ntasks x np, gamma ntasks; roots n x nv (as tracked, dehomogenized),
 *                    yfinal n x (nv + 2) (optional), resid n (optional, row-scaled residual) */
int or_num_plugins(void);
int or_plugin_info(int system, int* nv, int* np);
int or_plugin_rows(int system, const double* Y, const double* q, const double* dq, double* M, double* F);
int or_plugin_start(int system, const or_config* c, uint64_t seed, uint64_t stream, double* spt, double* spm);
int or_plugin_batch(int system, const or_config* c, uint64_t seed, const uint64_t* streams, int64_t n, int ntasks,
                    const int64_t* task_start, const double* fpm, const double* gamma, double* roots, int* codes,
                    double* yfinal, double* resid, int nthreads);
void or_philox_block(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
double or_uniform01(uint64_t seed, uint64_t stream, uint64_t index);

#endif
