// GENERATED by finite_root_generation_gb300/gen/gen_plugins.py from the modules in
// finite_root_generation_gb300/systems -- do not edit.
//
// System plug-ins for the one-thread-per-path tracker: the homogenized equations'
// rows of the homotopy Jacobian (columns Z, Z0, then the t column dF/dq . dq/dt) and
// the finite-root-generation start (random unknowns and free parameters, then the
// parameters that make the random point an exact root).
#pragma once

#include "frg_device.cuh"

namespace frg {

// ---- system 1: conic2 (2 unknowns, 12 parameters)
// rows(): 48 complex mul, 32 complex add/sub, 3 real x complex
struct Sys_conic2 {
  static constexpr int ID = 1;
  static constexpr int NV = 2;
  static constexpr int NP = 12;
  static constexpr int NS = 2;
  static constexpr int ROWS_CMUL = 48, ROWS_CADD = 32, ROWS_SMUL = 3;
  template <typename T, int LD>
  __device__ static void rows(const cx<T>* Y, const cx<T>* q, const cx<T>* dq, cx<T>* M, cx<T>* F) {
    const cx<T> u_x = Y[0];
    const cx<T> u_y = Y[1];
    const cx<T> u_Z0 = Y[2];
    const cx<T> p_a1 = q[0];
    const cx<T> dp_a1 = dq[0];
    const cx<T> p_b1 = q[1];
    const cx<T> dp_b1 = dq[1];
    const cx<T> p_c1 = q[2];
    const cx<T> dp_c1 = dq[2];
    const cx<T> p_d1 = q[3];
    const cx<T> dp_d1 = dq[3];
    const cx<T> p_e1 = q[4];
    const cx<T> dp_e1 = dq[4];
    const cx<T> p_f1 = q[5];
    const cx<T> dp_f1 = dq[5];
    const cx<T> p_a2 = q[6];
    const cx<T> dp_a2 = dq[6];
    const cx<T> p_b2 = q[7];
    const cx<T> dp_b2 = dq[7];
    const cx<T> p_c2 = q[8];
    const cx<T> dp_c2 = dq[8];
    const cx<T> p_d2 = q[9];
    const cx<T> dp_d2 = dq[9];
    const cx<T> p_e2 = q[10];
    const cx<T> dp_e2 = dq[10];
    const cx<T> p_f2 = q[11];
    const cx<T> dp_f2 = dq[11];
    const cx<T> r_0 = (u_Z0 * p_d1);
    const cx<T> r_1 = (p_b1 * u_y);
    const cx<T> r_2 = (T(2.0) * (u_x));
    const cx<T> r_3 = (u_Z0 * p_e1);
    const cx<T> r_4 = (T(2.0) * (u_y));
    const cx<T> r_5 = (T(2.0) * (u_Z0));
    const cx<T> r_6 = (u_Z0 * u_x);
    const cx<T> r_7 = (u_Z0 * u_y);
    const cx<T> r_8 = (u_x * u_y);
    const cx<T> r_9 = (u_Z0 * u_Z0);
    const cx<T> r_10 = (u_x * u_x);
    const cx<T> r_11 = (u_y * u_y);
    const cx<T> r_12 = (u_Z0 * p_d2);
    const cx<T> r_13 = (p_b2 * u_y);
    const cx<T> r_14 = (u_Z0 * p_e2);
    M[0 * LD + 0] = (r_0 + r_1 + (p_a1 * r_2));
    M[0 * LD + 1] = (r_3 + (p_b1 * u_x) + (p_c1 * r_4));
    M[0 * LD + 2] = ((p_d1 * u_x) + (p_e1 * u_y) + (p_f1 * r_5));
    M[0 * LD + 3] = ((dp_a1 * r_10) + (dp_b1 * r_8) + (dp_c1 * r_11) + (dp_d1 * r_6) + (dp_e1 * r_7) + (dp_f1 * r_9));
    M[1 * LD + 0] = (r_12 + r_13 + (p_a2 * r_2));
    M[1 * LD + 1] = (r_14 + (p_b2 * u_x) + (p_c2 * r_4));
    M[1 * LD + 2] = ((p_d2 * u_x) + (p_e2 * u_y) + (p_f2 * r_5));
    M[1 * LD + 3] = ((dp_a2 * r_10) + (dp_b2 * r_8) + (dp_c2 * r_11) + (dp_d2 * r_6) + (dp_e2 * r_7) + (dp_f2 * r_9));
    if (F) {
      F[0] = ((p_a1 * r_10) + (p_c1 * r_11) + (p_f1 * r_9) + (r_0 * u_x) + (r_1 * u_x) + (r_3 * u_y));
      F[1] = ((p_a2 * r_10) + (p_c2 * r_11) + (p_f2 * r_9) + (r_12 * u_x) + (r_13 * u_x) + (r_14 * u_y));
    }
  }
  __device__ static void start(Rng& rng, int dist, double range, cd* z, cd* q) {
    typedef double T;
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[0] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[1] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[0] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[1] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[2] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[3] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[4] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[6] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[7] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[8] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[9] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[10] = cd(re, im); }
    const cx<T> u_x = z[0];
    const cx<T> u_y = z[1];
    const cx<T> p_a1 = q[0];
    const cx<T> p_b1 = q[1];
    const cx<T> p_c1 = q[2];
    const cx<T> p_d1 = q[3];
    const cx<T> p_e1 = q[4];
    const cx<T> p_a2 = q[6];
    const cx<T> p_b2 = q[7];
    const cx<T> p_c2 = q[8];
    const cx<T> p_d2 = q[9];
    const cx<T> p_e2 = q[10];
    const cx<T> s_0 = (u_x * u_y);
    const cx<T> s_1 = (u_x * u_x);
    const cx<T> s_2 = (u_y * u_y);
    cx<T> A[4], b[2], s[2];
    A[0] = cx<T>(T(1.0));
    A[1] = cx<T>(T(0));
    A[2] = cx<T>(T(0));
    A[3] = cx<T>(T(1.0));
    b[0] = ((-(p_a1 * s_1)) - (p_b1 * s_0) - (p_c1 * s_2) - (p_d1 * u_x) - (p_e1 * u_y));
    b[1] = ((-(p_a2 * s_1)) - (p_b2 * s_0) - (p_c2 * s_2) - (p_d2 * u_x) - (p_e2 * u_y));
    small_solve<2>(A, b, s);
    q[5] = s[0];
    q[11] = s[1];
  }
  __device__ static void canonical(const cd* root, const cd*, cd* out) {
    for (int i = 0; i < NV; ++i) out[i] = root[i];
  }
};

// ---- system 2: burmester5 (5 unknowns, 20 parameters)
// rows(): 158 complex mul, 101 complex add/sub, 5 real x complex
struct Sys_burmester5 {
  static constexpr int ID = 2;
  static constexpr int NV = 5;
  static constexpr int NP = 20;
  static constexpr int NS = 5;
  static constexpr int ROWS_CMUL = 158, ROWS_CADD = 101, ROWS_SMUL = 5;
  template <typename T, int LD>
  __device__ static void rows(const cx<T>* Y, const cx<T>* q, const cx<T>* dq, cx<T>* M, cx<T>* F) {
    const cx<T> u_G = Y[0];
    const cx<T> u_Gc = Y[1];
    const cx<T> u_z = Y[2];
    const cx<T> u_zc = Y[3];
    const cx<T> u_R = Y[4];
    const cx<T> u_Z0 = Y[5];
    const cx<T> p_d0 = q[0];
    const cx<T> dp_d0 = dq[0];
    const cx<T> p_d1 = q[1];
    const cx<T> dp_d1 = dq[1];
    const cx<T> p_d2 = q[2];
    const cx<T> dp_d2 = dq[2];
    const cx<T> p_d3 = q[3];
    const cx<T> dp_d3 = dq[3];
    const cx<T> p_d4 = q[4];
    const cx<T> dp_d4 = dq[4];
    const cx<T> p_dc0 = q[5];
    const cx<T> dp_dc0 = dq[5];
    const cx<T> p_dc1 = q[6];
    const cx<T> dp_dc1 = dq[6];
    const cx<T> p_dc2 = q[7];
    const cx<T> dp_dc2 = dq[7];
    const cx<T> p_dc3 = q[8];
    const cx<T> dp_dc3 = dq[8];
    const cx<T> p_dc4 = q[9];
    const cx<T> dp_dc4 = dq[9];
    const cx<T> p_T0 = q[10];
    const cx<T> dp_T0 = dq[10];
    const cx<T> p_T1 = q[11];
    const cx<T> dp_T1 = dq[11];
    const cx<T> p_T2 = q[12];
    const cx<T> dp_T2 = dq[12];
    const cx<T> p_T3 = q[13];
    const cx<T> dp_T3 = dq[13];
    const cx<T> p_T4 = q[14];
    const cx<T> dp_T4 = dq[14];
    const cx<T> p_Tc0 = q[15];
    const cx<T> dp_Tc0 = dq[15];
    const cx<T> p_Tc1 = q[16];
    const cx<T> dp_Tc1 = dq[16];
    const cx<T> p_Tc2 = q[17];
    const cx<T> dp_Tc2 = dq[17];
    const cx<T> p_Tc3 = q[18];
    const cx<T> dp_Tc3 = dq[18];
    const cx<T> p_Tc4 = q[19];
    const cx<T> dp_Tc4 = dq[19];
    const cx<T> r_0 = (-(u_Gc));
    const cx<T> r_1 = (p_Tc0 * u_zc);
    const cx<T> r_2 = (u_Z0 * p_dc0);
    const cx<T> r_3 = (r_0 + r_1 + r_2);
    const cx<T> r_4 = (-(u_G));
    const cx<T> r_5 = (p_T0 * u_z);
    const cx<T> r_6 = (u_Z0 * p_d0);
    const cx<T> r_7 = (r_4 + r_5 + r_6);
    const cx<T> r_8 = (-(u_Z0));
    const cx<T> r_9 = (p_Tc1 * u_zc);
    const cx<T> r_10 = (u_Z0 * p_dc1);
    const cx<T> r_11 = (r_0 + r_10 + r_9);
    const cx<T> r_12 = (p_T1 * u_z);
    const cx<T> r_13 = (u_Z0 * p_d1);
    const cx<T> r_14 = (r_12 + r_13 + r_4);
    const cx<T> r_15 = (p_Tc2 * u_zc);
    const cx<T> r_16 = (u_Z0 * p_dc2);
    const cx<T> r_17 = (r_0 + r_15 + r_16);
    const cx<T> r_18 = (p_T2 * u_z);
    const cx<T> r_19 = (u_Z0 * p_d2);
    const cx<T> r_20 = (r_18 + r_19 + r_4);
    const cx<T> r_21 = (p_Tc3 * u_zc);
    const cx<T> r_22 = (u_Z0 * p_dc3);
    const cx<T> r_23 = (r_0 + r_21 + r_22);
    const cx<T> r_24 = (p_T3 * u_z);
    const cx<T> r_25 = (u_Z0 * p_d3);
    const cx<T> r_26 = (r_24 + r_25 + r_4);
    const cx<T> r_27 = (p_Tc4 * u_zc);
    const cx<T> r_28 = (u_Z0 * p_dc4);
    const cx<T> r_29 = (r_0 + r_27 + r_28);
    const cx<T> r_30 = (p_T4 * u_z);
    const cx<T> r_31 = (u_Z0 * p_d4);
    const cx<T> r_32 = (r_30 + r_31 + r_4);
    const cx<T> r_33 = (u_Z0 * u_Z0);
    const cx<T> r_34 = ((u_G * u_Gc) - (u_R * u_Z0));
    M[0 * LD + 0] = (-(r_3));
    M[0 * LD + 1] = (-(r_7));
    M[0 * LD + 2] = (p_T0 * r_3);
    M[0 * LD + 3] = (p_Tc0 * r_7);
    M[0 * LD + 4] = r_8;
    M[0 * LD + 5] = ((-u_R) - (u_G * p_dc0) - (u_Gc * p_d0) + (p_T0 * p_dc0 * u_z) + (p_Tc0 * p_d0 * u_zc) + (T(2.0) * ((u_Z0 * p_d0 * p_dc0))));
    M[0 * LD + 6] = ((u_Z0 * dp_d0 * r_3) + (u_Z0 * dp_dc0 * r_7) + (dp_T0 * r_3 * u_z) + (dp_Tc0 * r_7 * u_zc));
    M[1 * LD + 0] = (-(r_11));
    M[1 * LD + 1] = (-(r_14));
    M[1 * LD + 2] = (p_T1 * r_11);
    M[1 * LD + 3] = (p_Tc1 * r_14);
    M[1 * LD + 4] = r_8;
    M[1 * LD + 5] = ((-u_R) - (u_G * p_dc1) - (u_Gc * p_d1) + (p_T1 * p_dc1 * u_z) + (p_Tc1 * p_d1 * u_zc) + (T(2.0) * ((u_Z0 * p_d1 * p_dc1))));
    M[1 * LD + 6] = ((u_Z0 * dp_d1 * r_11) + (u_Z0 * dp_dc1 * r_14) + (dp_T1 * r_11 * u_z) + (dp_Tc1 * r_14 * u_zc));
    M[2 * LD + 0] = (-(r_17));
    M[2 * LD + 1] = (-(r_20));
    M[2 * LD + 2] = (p_T2 * r_17);
    M[2 * LD + 3] = (p_Tc2 * r_20);
    M[2 * LD + 4] = r_8;
    M[2 * LD + 5] = ((-u_R) - (u_G * p_dc2) - (u_Gc * p_d2) + (p_T2 * p_dc2 * u_z) + (p_Tc2 * p_d2 * u_zc) + (T(2.0) * ((u_Z0 * p_d2 * p_dc2))));
    M[2 * LD + 6] = ((u_Z0 * dp_d2 * r_17) + (u_Z0 * dp_dc2 * r_20) + (dp_T2 * r_17 * u_z) + (dp_Tc2 * r_20 * u_zc));
    M[3 * LD + 0] = (-(r_23));
    M[3 * LD + 1] = (-(r_26));
    M[3 * LD + 2] = (p_T3 * r_23);
    M[3 * LD + 3] = (p_Tc3 * r_26);
    M[3 * LD + 4] = r_8;
    M[3 * LD + 5] = ((-u_R) - (u_G * p_dc3) - (u_Gc * p_d3) + (p_T3 * p_dc3 * u_z) + (p_Tc3 * p_d3 * u_zc) + (T(2.0) * ((u_Z0 * p_d3 * p_dc3))));
    M[3 * LD + 6] = ((u_Z0 * dp_d3 * r_23) + (u_Z0 * dp_dc3 * r_26) + (dp_T3 * r_23 * u_z) + (dp_Tc3 * r_26 * u_zc));
    M[4 * LD + 0] = (-(r_29));
    M[4 * LD + 1] = (-(r_32));
    M[4 * LD + 2] = (p_T4 * r_29);
    M[4 * LD + 3] = (p_Tc4 * r_32);
    M[4 * LD + 4] = r_8;
    M[4 * LD + 5] = ((-u_R) - (u_G * p_dc4) - (u_Gc * p_d4) + (p_T4 * p_dc4 * u_z) + (p_Tc4 * p_d4 * u_zc) + (T(2.0) * ((u_Z0 * p_d4 * p_dc4))));
    M[4 * LD + 6] = ((u_Z0 * dp_d4 * r_29) + (u_Z0 * dp_dc4 * r_32) + (dp_T4 * r_29 * u_z) + (dp_Tc4 * r_32 * u_zc));
    if (F) {
      F[0] = (r_34 + (r_1 * r_5) + (r_1 * r_6) + (r_2 * r_5) - (u_G * r_1) - (u_G * r_2) - (u_Gc * r_5) - (u_Gc * r_6) + (p_d0 * p_dc0 * r_33));
      F[1] = (r_34 + (r_10 * r_12) + (r_12 * r_9) + (r_13 * r_9) - (u_G * r_10) - (u_G * r_9) - (u_Gc * r_12) - (u_Gc * r_13) + (p_d1 * p_dc1 * r_33));
      F[2] = (r_34 + (r_15 * r_18) + (r_15 * r_19) + (r_16 * r_18) - (u_G * r_15) - (u_G * r_16) - (u_Gc * r_18) - (u_Gc * r_19) + (p_d2 * p_dc2 * r_33));
      F[3] = (r_34 + (r_21 * r_24) + (r_21 * r_25) + (r_22 * r_24) - (u_G * r_21) - (u_G * r_22) - (u_Gc * r_24) - (u_Gc * r_25) + (p_d3 * p_dc3 * r_33));
      F[4] = (r_34 + (r_27 * r_30) + (r_27 * r_31) + (r_28 * r_30) - (u_G * r_27) - (u_G * r_28) - (u_Gc * r_30) - (u_Gc * r_31) + (p_d4 * p_dc4 * r_33));
    }
  }
  __device__ static void start(Rng& rng, int dist, double range, cd* z, cd* q) {
    typedef double T;
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[0] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[1] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[2] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[3] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); z[4] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[5] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[6] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[7] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[8] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[9] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[10] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[11] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[12] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[13] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[14] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[15] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[16] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[17] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[18] = cd(re, im); }
    { const double re = start_value(rng, dist, range); const double im = start_value(rng, dist, range); q[19] = cd(re, im); }
    const cx<T> u_G = z[0];
    const cx<T> u_Gc = z[1];
    const cx<T> u_z = z[2];
    const cx<T> u_zc = z[3];
    const cx<T> u_R = z[4];
    const cx<T> p_dc0 = q[5];
    const cx<T> p_dc1 = q[6];
    const cx<T> p_dc2 = q[7];
    const cx<T> p_dc3 = q[8];
    const cx<T> p_dc4 = q[9];
    const cx<T> p_T0 = q[10];
    const cx<T> p_T1 = q[11];
    const cx<T> p_T2 = q[12];
    const cx<T> p_T3 = q[13];
    const cx<T> p_T4 = q[14];
    const cx<T> p_Tc0 = q[15];
    const cx<T> p_Tc1 = q[16];
    const cx<T> p_Tc2 = q[17];
    const cx<T> p_Tc3 = q[18];
    const cx<T> p_Tc4 = q[19];
    const cx<T> s_0 = (-(u_Gc));
    const cx<T> s_1 = (p_Tc0 * u_zc);
    const cx<T> s_2 = (p_Tc1 * u_zc);
    const cx<T> s_3 = (p_Tc2 * u_zc);
    const cx<T> s_4 = (p_Tc3 * u_zc);
    const cx<T> s_5 = (p_Tc4 * u_zc);
    const cx<T> s_6 = (u_R - (u_G * u_Gc));
    cx<T> A[25], b[5], s[5];
    A[0] = (p_dc0 + s_0 + s_1);
    A[1] = cx<T>(T(0));
    A[2] = cx<T>(T(0));
    A[3] = cx<T>(T(0));
    A[4] = cx<T>(T(0));
    A[5] = cx<T>(T(0));
    A[6] = (p_dc1 + s_0 + s_2);
    A[7] = cx<T>(T(0));
    A[8] = cx<T>(T(0));
    A[9] = cx<T>(T(0));
    A[10] = cx<T>(T(0));
    A[11] = cx<T>(T(0));
    A[12] = (p_dc2 + s_0 + s_3);
    A[13] = cx<T>(T(0));
    A[14] = cx<T>(T(0));
    A[15] = cx<T>(T(0));
    A[16] = cx<T>(T(0));
    A[17] = cx<T>(T(0));
    A[18] = (p_dc3 + s_0 + s_4);
    A[19] = cx<T>(T(0));
    A[20] = cx<T>(T(0));
    A[21] = cx<T>(T(0));
    A[22] = cx<T>(T(0));
    A[23] = cx<T>(T(0));
    A[24] = (p_dc4 + s_0 + s_5);
    b[0] = (s_6 + (u_G * p_dc0) + (u_G * s_1) + (u_Gc * p_T0 * u_z) - (p_T0 * p_dc0 * u_z) - (p_T0 * p_Tc0 * u_z * u_zc));
    b[1] = (s_6 + (u_G * p_dc1) + (u_G * s_2) + (u_Gc * p_T1 * u_z) - (p_T1 * p_dc1 * u_z) - (p_T1 * p_Tc1 * u_z * u_zc));
    b[2] = (s_6 + (u_G * p_dc2) + (u_G * s_3) + (u_Gc * p_T2 * u_z) - (p_T2 * p_dc2 * u_z) - (p_T2 * p_Tc2 * u_z * u_zc));
    b[3] = (s_6 + (u_G * p_dc3) + (u_G * s_4) + (u_Gc * p_T3 * u_z) - (p_T3 * p_dc3 * u_z) - (p_T3 * p_Tc3 * u_z * u_zc));
    b[4] = (s_6 + (u_G * p_dc4) + (u_G * s_5) + (u_Gc * p_T4 * u_z) - (p_T4 * p_dc4 * u_z) - (p_T4 * p_Tc4 * u_z * u_zc));
    small_solve<5>(A, b, s);
    q[0] = s[0];
    q[1] = s[1];
    q[2] = s[2];
    q[3] = s[3];
    q[4] = s[4];
  }
  __device__ static void canonical(const cd* root, const cd*, cd* out) {
    for (int i = 0; i < NV; ++i) out[i] = root[i];
  }
};

}  // namespace frg

// X(id, name, struct) for every plug-in
#define FRG_PLUGIN_LIST(X) \
  X(1, "conic2", frg::Sys_conic2) \
  X(2, "burmester5", frg::Sys_burmester5) \

#define FRG_NUM_PLUGINS 2
