/* GENERATED by finite_root_generation_gb300/gen/gen_plugins.py from the modules in
 * finite_root_generation_gb300/systems -- do not edit.
 *
 * ORACLE TEST INFRASTRUCTURE: the plug-in systems' rows and starts for the oracle's
 * tracker (included by frg_oracle.c, which defines cd, mk, cadd, csub, cmul, cscal,
 * rng_t, start_draw and small_solve). */

/* ---- system 1: conic2 (2 unknowns, 12 parameters) */
static void plug_conic2_rows(const cd* Y, const cd* q, const cd* dq, cd* M, int ld, cd* F) {
  const cd u_x = Y[0];
  const cd u_y = Y[1];
  const cd u_Z0 = Y[2];
  const cd p_a1 = q[0];
  const cd dp_a1 = dq[0];
  const cd p_b1 = q[1];
  const cd dp_b1 = dq[1];
  const cd p_c1 = q[2];
  const cd dp_c1 = dq[2];
  const cd p_d1 = q[3];
  const cd dp_d1 = dq[3];
  const cd p_e1 = q[4];
  const cd dp_e1 = dq[4];
  const cd p_f1 = q[5];
  const cd dp_f1 = dq[5];
  const cd p_a2 = q[6];
  const cd dp_a2 = dq[6];
  const cd p_b2 = q[7];
  const cd dp_b2 = dq[7];
  const cd p_c2 = q[8];
  const cd dp_c2 = dq[8];
  const cd p_d2 = q[9];
  const cd dp_d2 = dq[9];
  const cd p_e2 = q[10];
  const cd dp_e2 = dq[10];
  const cd p_f2 = q[11];
  const cd dp_f2 = dq[11];
  const cd r_0 = cmul(u_Z0, p_d1);
  const cd r_1 = cmul(p_b1, u_y);
  const cd r_2 = cscal(2.0, u_x);
  const cd r_3 = cmul(u_Z0, p_e1);
  const cd r_4 = cscal(2.0, u_y);
  const cd r_5 = cscal(2.0, u_Z0);
  const cd r_6 = cmul(u_Z0, u_x);
  const cd r_7 = cmul(u_Z0, u_y);
  const cd r_8 = cmul(u_x, u_y);
  const cd r_9 = cmul(u_Z0, u_Z0);
  const cd r_10 = cmul(u_x, u_x);
  const cd r_11 = cmul(u_y, u_y);
  const cd r_12 = cmul(u_Z0, p_d2);
  const cd r_13 = cmul(p_b2, u_y);
  const cd r_14 = cmul(u_Z0, p_e2);
  M[0 * ld + 0] = cadd(cadd(r_0, r_1), cmul(p_a1, r_2));
  M[0 * ld + 1] = cadd(cadd(r_3, cmul(p_b1, u_x)), cmul(p_c1, r_4));
  M[0 * ld + 2] = cadd(cadd(cmul(p_d1, u_x), cmul(p_e1, u_y)), cmul(p_f1, r_5));
  M[0 * ld + 3] = cadd(cadd(cadd(cadd(cadd(cmul(dp_a1, r_10), cmul(dp_b1, r_8)), cmul(dp_c1, r_11)), cmul(dp_d1, r_6)), cmul(dp_e1, r_7)), cmul(dp_f1, r_9));
  M[1 * ld + 0] = cadd(cadd(r_12, r_13), cmul(p_a2, r_2));
  M[1 * ld + 1] = cadd(cadd(r_14, cmul(p_b2, u_x)), cmul(p_c2, r_4));
  M[1 * ld + 2] = cadd(cadd(cmul(p_d2, u_x), cmul(p_e2, u_y)), cmul(p_f2, r_5));
  M[1 * ld + 3] = cadd(cadd(cadd(cadd(cadd(cmul(dp_a2, r_10), cmul(dp_b2, r_8)), cmul(dp_c2, r_11)), cmul(dp_d2, r_6)), cmul(dp_e2, r_7)), cmul(dp_f2, r_9));
  if (F) {
    F[0] = cadd(cadd(cadd(cadd(cadd(cmul(p_a1, r_10), cmul(p_c1, r_11)), cmul(p_f1, r_9)), cmul(r_0, u_x)), cmul(r_1, u_x)), cmul(r_3, u_y));
    F[1] = cadd(cadd(cadd(cadd(cadd(cmul(p_a2, r_10), cmul(p_c2, r_11)), cmul(p_f2, r_9)), cmul(r_12, u_x)), cmul(r_13, u_x)), cmul(r_14, u_y));
  }
}
static void plug_conic2_start(const or_config* c, rng_t* r, cd* z, cd* q) {
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[0] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[1] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[0] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[1] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[2] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[3] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[4] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[6] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[7] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[8] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[9] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[10] = mk(re, im); }
  const cd u_x = z[0];
  const cd u_y = z[1];
  const cd p_a1 = q[0];
  const cd p_b1 = q[1];
  const cd p_c1 = q[2];
  const cd p_d1 = q[3];
  const cd p_e1 = q[4];
  const cd p_a2 = q[6];
  const cd p_b2 = q[7];
  const cd p_c2 = q[8];
  const cd p_d2 = q[9];
  const cd p_e2 = q[10];
  const cd s_0 = cmul(u_x, u_y);
  const cd s_1 = cmul(u_x, u_x);
  const cd s_2 = cmul(u_y, u_y);
  cd A[4], b[2], s[2];
  A[0] = mk(1.0, 0.0);
  A[1] = mk(0.0, 0.0);
  A[2] = mk(0.0, 0.0);
  A[3] = mk(1.0, 0.0);
  b[0] = csub(csub(csub(csub(cscal(-1.0, cmul(p_a1, s_1)), cmul(p_b1, s_0)), cmul(p_c1, s_2)), cmul(p_d1, u_x)), cmul(p_e1, u_y));
  b[1] = csub(csub(csub(csub(cscal(-1.0, cmul(p_a2, s_1)), cmul(p_b2, s_0)), cmul(p_c2, s_2)), cmul(p_d2, u_x)), cmul(p_e2, u_y));
  small_solve(2, A, b, s);
  q[5] = s[0];
  q[11] = s[1];
}

/* ---- system 2: burmester5 (5 unknowns, 20 parameters) */
static void plug_burmester5_rows(const cd* Y, const cd* q, const cd* dq, cd* M, int ld, cd* F) {
  const cd u_G = Y[0];
  const cd u_Gc = Y[1];
  const cd u_z = Y[2];
  const cd u_zc = Y[3];
  const cd u_R = Y[4];
  const cd u_Z0 = Y[5];
  const cd p_d0 = q[0];
  const cd dp_d0 = dq[0];
  const cd p_d1 = q[1];
  const cd dp_d1 = dq[1];
  const cd p_d2 = q[2];
  const cd dp_d2 = dq[2];
  const cd p_d3 = q[3];
  const cd dp_d3 = dq[3];
  const cd p_d4 = q[4];
  const cd dp_d4 = dq[4];
  const cd p_dc0 = q[5];
  const cd dp_dc0 = dq[5];
  const cd p_dc1 = q[6];
  const cd dp_dc1 = dq[6];
  const cd p_dc2 = q[7];
  const cd dp_dc2 = dq[7];
  const cd p_dc3 = q[8];
  const cd dp_dc3 = dq[8];
  const cd p_dc4 = q[9];
  const cd dp_dc4 = dq[9];
  const cd p_T0 = q[10];
  const cd dp_T0 = dq[10];
  const cd p_T1 = q[11];
  const cd dp_T1 = dq[11];
  const cd p_T2 = q[12];
  const cd dp_T2 = dq[12];
  const cd p_T3 = q[13];
  const cd dp_T3 = dq[13];
  const cd p_T4 = q[14];
  const cd dp_T4 = dq[14];
  const cd p_Tc0 = q[15];
  const cd dp_Tc0 = dq[15];
  const cd p_Tc1 = q[16];
  const cd dp_Tc1 = dq[16];
  const cd p_Tc2 = q[17];
  const cd dp_Tc2 = dq[17];
  const cd p_Tc3 = q[18];
  const cd dp_Tc3 = dq[18];
  const cd p_Tc4 = q[19];
  const cd dp_Tc4 = dq[19];
  const cd r_0 = cscal(-1.0, u_Gc);
  const cd r_1 = cmul(p_Tc0, u_zc);
  const cd r_2 = cmul(u_Z0, p_dc0);
  const cd r_3 = cadd(cadd(r_0, r_1), r_2);
  const cd r_4 = cscal(-1.0, u_G);
  const cd r_5 = cmul(p_T0, u_z);
  const cd r_6 = cmul(u_Z0, p_d0);
  const cd r_7 = cadd(cadd(r_4, r_5), r_6);
  const cd r_8 = cscal(-1.0, u_Z0);
  const cd r_9 = cmul(p_Tc1, u_zc);
  const cd r_10 = cmul(u_Z0, p_dc1);
  const cd r_11 = cadd(cadd(r_0, r_10), r_9);
  const cd r_12 = cmul(p_T1, u_z);
  const cd r_13 = cmul(u_Z0, p_d1);
  const cd r_14 = cadd(cadd(r_12, r_13), r_4);
  const cd r_15 = cmul(p_Tc2, u_zc);
  const cd r_16 = cmul(u_Z0, p_dc2);
  const cd r_17 = cadd(cadd(r_0, r_15), r_16);
  const cd r_18 = cmul(p_T2, u_z);
  const cd r_19 = cmul(u_Z0, p_d2);
  const cd r_20 = cadd(cadd(r_18, r_19), r_4);
  const cd r_21 = cmul(p_Tc3, u_zc);
  const cd r_22 = cmul(u_Z0, p_dc3);
  const cd r_23 = cadd(cadd(r_0, r_21), r_22);
  const cd r_24 = cmul(p_T3, u_z);
  const cd r_25 = cmul(u_Z0, p_d3);
  const cd r_26 = cadd(cadd(r_24, r_25), r_4);
  const cd r_27 = cmul(p_Tc4, u_zc);
  const cd r_28 = cmul(u_Z0, p_dc4);
  const cd r_29 = cadd(cadd(r_0, r_27), r_28);
  const cd r_30 = cmul(p_T4, u_z);
  const cd r_31 = cmul(u_Z0, p_d4);
  const cd r_32 = cadd(cadd(r_30, r_31), r_4);
  const cd r_33 = cmul(u_Z0, u_Z0);
  const cd r_34 = csub(cmul(u_G, u_Gc), cmul(u_R, u_Z0));
  M[0 * ld + 0] = cscal(-1.0, r_3);
  M[0 * ld + 1] = cscal(-1.0, r_7);
  M[0 * ld + 2] = cmul(p_T0, r_3);
  M[0 * ld + 3] = cmul(p_Tc0, r_7);
  M[0 * ld + 4] = r_8;
  M[0 * ld + 5] = cadd(cadd(cadd(csub(csub(cscal(-1.0, u_R), cmul(u_G, p_dc0)), cmul(u_Gc, p_d0)), cmul(p_T0, cmul(p_dc0, u_z))), cmul(p_Tc0, cmul(p_d0, u_zc))), cscal(2.0, cmul(u_Z0, cmul(p_d0, p_dc0))));
  M[0 * ld + 6] = cadd(cadd(cadd(cmul(u_Z0, cmul(dp_d0, r_3)), cmul(u_Z0, cmul(dp_dc0, r_7))), cmul(dp_T0, cmul(r_3, u_z))), cmul(dp_Tc0, cmul(r_7, u_zc)));
  M[1 * ld + 0] = cscal(-1.0, r_11);
  M[1 * ld + 1] = cscal(-1.0, r_14);
  M[1 * ld + 2] = cmul(p_T1, r_11);
  M[1 * ld + 3] = cmul(p_Tc1, r_14);
  M[1 * ld + 4] = r_8;
  M[1 * ld + 5] = cadd(cadd(cadd(csub(csub(cscal(-1.0, u_R), cmul(u_G, p_dc1)), cmul(u_Gc, p_d1)), cmul(p_T1, cmul(p_dc1, u_z))), cmul(p_Tc1, cmul(p_d1, u_zc))), cscal(2.0, cmul(u_Z0, cmul(p_d1, p_dc1))));
  M[1 * ld + 6] = cadd(cadd(cadd(cmul(u_Z0, cmul(dp_d1, r_11)), cmul(u_Z0, cmul(dp_dc1, r_14))), cmul(dp_T1, cmul(r_11, u_z))), cmul(dp_Tc1, cmul(r_14, u_zc)));
  M[2 * ld + 0] = cscal(-1.0, r_17);
  M[2 * ld + 1] = cscal(-1.0, r_20);
  M[2 * ld + 2] = cmul(p_T2, r_17);
  M[2 * ld + 3] = cmul(p_Tc2, r_20);
  M[2 * ld + 4] = r_8;
  M[2 * ld + 5] = cadd(cadd(cadd(csub(csub(cscal(-1.0, u_R), cmul(u_G, p_dc2)), cmul(u_Gc, p_d2)), cmul(p_T2, cmul(p_dc2, u_z))), cmul(p_Tc2, cmul(p_d2, u_zc))), cscal(2.0, cmul(u_Z0, cmul(p_d2, p_dc2))));
  M[2 * ld + 6] = cadd(cadd(cadd(cmul(u_Z0, cmul(dp_d2, r_17)), cmul(u_Z0, cmul(dp_dc2, r_20))), cmul(dp_T2, cmul(r_17, u_z))), cmul(dp_Tc2, cmul(r_20, u_zc)));
  M[3 * ld + 0] = cscal(-1.0, r_23);
  M[3 * ld + 1] = cscal(-1.0, r_26);
  M[3 * ld + 2] = cmul(p_T3, r_23);
  M[3 * ld + 3] = cmul(p_Tc3, r_26);
  M[3 * ld + 4] = r_8;
  M[3 * ld + 5] = cadd(cadd(cadd(csub(csub(cscal(-1.0, u_R), cmul(u_G, p_dc3)), cmul(u_Gc, p_d3)), cmul(p_T3, cmul(p_dc3, u_z))), cmul(p_Tc3, cmul(p_d3, u_zc))), cscal(2.0, cmul(u_Z0, cmul(p_d3, p_dc3))));
  M[3 * ld + 6] = cadd(cadd(cadd(cmul(u_Z0, cmul(dp_d3, r_23)), cmul(u_Z0, cmul(dp_dc3, r_26))), cmul(dp_T3, cmul(r_23, u_z))), cmul(dp_Tc3, cmul(r_26, u_zc)));
  M[4 * ld + 0] = cscal(-1.0, r_29);
  M[4 * ld + 1] = cscal(-1.0, r_32);
  M[4 * ld + 2] = cmul(p_T4, r_29);
  M[4 * ld + 3] = cmul(p_Tc4, r_32);
  M[4 * ld + 4] = r_8;
  M[4 * ld + 5] = cadd(cadd(cadd(csub(csub(cscal(-1.0, u_R), cmul(u_G, p_dc4)), cmul(u_Gc, p_d4)), cmul(p_T4, cmul(p_dc4, u_z))), cmul(p_Tc4, cmul(p_d4, u_zc))), cscal(2.0, cmul(u_Z0, cmul(p_d4, p_dc4))));
  M[4 * ld + 6] = cadd(cadd(cadd(cmul(u_Z0, cmul(dp_d4, r_29)), cmul(u_Z0, cmul(dp_dc4, r_32))), cmul(dp_T4, cmul(r_29, u_z))), cmul(dp_Tc4, cmul(r_32, u_zc)));
  if (F) {
    F[0] = cadd(csub(csub(csub(csub(cadd(cadd(cadd(r_34, cmul(r_1, r_5)), cmul(r_1, r_6)), cmul(r_2, r_5)), cmul(u_G, r_1)), cmul(u_G, r_2)), cmul(u_Gc, r_5)), cmul(u_Gc, r_6)), cmul(p_d0, cmul(p_dc0, r_33)));
    F[1] = cadd(csub(csub(csub(csub(cadd(cadd(cadd(r_34, cmul(r_10, r_12)), cmul(r_12, r_9)), cmul(r_13, r_9)), cmul(u_G, r_10)), cmul(u_G, r_9)), cmul(u_Gc, r_12)), cmul(u_Gc, r_13)), cmul(p_d1, cmul(p_dc1, r_33)));
    F[2] = cadd(csub(csub(csub(csub(cadd(cadd(cadd(r_34, cmul(r_15, r_18)), cmul(r_15, r_19)), cmul(r_16, r_18)), cmul(u_G, r_15)), cmul(u_G, r_16)), cmul(u_Gc, r_18)), cmul(u_Gc, r_19)), cmul(p_d2, cmul(p_dc2, r_33)));
    F[3] = cadd(csub(csub(csub(csub(cadd(cadd(cadd(r_34, cmul(r_21, r_24)), cmul(r_21, r_25)), cmul(r_22, r_24)), cmul(u_G, r_21)), cmul(u_G, r_22)), cmul(u_Gc, r_24)), cmul(u_Gc, r_25)), cmul(p_d3, cmul(p_dc3, r_33)));
    F[4] = cadd(csub(csub(csub(csub(cadd(cadd(cadd(r_34, cmul(r_27, r_30)), cmul(r_27, r_31)), cmul(r_28, r_30)), cmul(u_G, r_27)), cmul(u_G, r_28)), cmul(u_Gc, r_30)), cmul(u_Gc, r_31)), cmul(p_d4, cmul(p_dc4, r_33)));
  }
}
static void plug_burmester5_start(const or_config* c, rng_t* r, cd* z, cd* q) {
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[0] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[1] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[2] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[3] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); z[4] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[5] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[6] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[7] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[8] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[9] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[10] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[11] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[12] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[13] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[14] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[15] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[16] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[17] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[18] = mk(re, im); }
  { const double re = start_draw(c, r); const double im = start_draw(c, r); q[19] = mk(re, im); }
  const cd u_G = z[0];
  const cd u_Gc = z[1];
  const cd u_z = z[2];
  const cd u_zc = z[3];
  const cd u_R = z[4];
  const cd p_dc0 = q[5];
  const cd p_dc1 = q[6];
  const cd p_dc2 = q[7];
  const cd p_dc3 = q[8];
  const cd p_dc4 = q[9];
  const cd p_T0 = q[10];
  const cd p_T1 = q[11];
  const cd p_T2 = q[12];
  const cd p_T3 = q[13];
  const cd p_T4 = q[14];
  const cd p_Tc0 = q[15];
  const cd p_Tc1 = q[16];
  const cd p_Tc2 = q[17];
  const cd p_Tc3 = q[18];
  const cd p_Tc4 = q[19];
  const cd s_0 = cscal(-1.0, u_Gc);
  const cd s_1 = cmul(p_Tc0, u_zc);
  const cd s_2 = cmul(p_Tc1, u_zc);
  const cd s_3 = cmul(p_Tc2, u_zc);
  const cd s_4 = cmul(p_Tc3, u_zc);
  const cd s_5 = cmul(p_Tc4, u_zc);
  const cd s_6 = csub(u_R, cmul(u_G, u_Gc));
  cd A[25], b[5], s[5];
  A[0] = cadd(cadd(p_dc0, s_0), s_1);
  A[1] = mk(0.0, 0.0);
  A[2] = mk(0.0, 0.0);
  A[3] = mk(0.0, 0.0);
  A[4] = mk(0.0, 0.0);
  A[5] = mk(0.0, 0.0);
  A[6] = cadd(cadd(p_dc1, s_0), s_2);
  A[7] = mk(0.0, 0.0);
  A[8] = mk(0.0, 0.0);
  A[9] = mk(0.0, 0.0);
  A[10] = mk(0.0, 0.0);
  A[11] = mk(0.0, 0.0);
  A[12] = cadd(cadd(p_dc2, s_0), s_3);
  A[13] = mk(0.0, 0.0);
  A[14] = mk(0.0, 0.0);
  A[15] = mk(0.0, 0.0);
  A[16] = mk(0.0, 0.0);
  A[17] = mk(0.0, 0.0);
  A[18] = cadd(cadd(p_dc3, s_0), s_4);
  A[19] = mk(0.0, 0.0);
  A[20] = mk(0.0, 0.0);
  A[21] = mk(0.0, 0.0);
  A[22] = mk(0.0, 0.0);
  A[23] = mk(0.0, 0.0);
  A[24] = cadd(cadd(p_dc4, s_0), s_5);
  b[0] = csub(csub(cadd(cadd(cadd(s_6, cmul(u_G, p_dc0)), cmul(u_G, s_1)), cmul(u_Gc, cmul(p_T0, u_z))), cmul(p_T0, cmul(p_dc0, u_z))), cmul(p_T0, cmul(p_Tc0, cmul(u_z, u_zc))));
  b[1] = csub(csub(cadd(cadd(cadd(s_6, cmul(u_G, p_dc1)), cmul(u_G, s_2)), cmul(u_Gc, cmul(p_T1, u_z))), cmul(p_T1, cmul(p_dc1, u_z))), cmul(p_T1, cmul(p_Tc1, cmul(u_z, u_zc))));
  b[2] = csub(csub(cadd(cadd(cadd(s_6, cmul(u_G, p_dc2)), cmul(u_G, s_3)), cmul(u_Gc, cmul(p_T2, u_z))), cmul(p_T2, cmul(p_dc2, u_z))), cmul(p_T2, cmul(p_Tc2, cmul(u_z, u_zc))));
  b[3] = csub(csub(cadd(cadd(cadd(s_6, cmul(u_G, p_dc3)), cmul(u_G, s_4)), cmul(u_Gc, cmul(p_T3, u_z))), cmul(p_T3, cmul(p_dc3, u_z))), cmul(p_T3, cmul(p_Tc3, cmul(u_z, u_zc))));
  b[4] = csub(csub(cadd(cadd(cadd(s_6, cmul(u_G, p_dc4)), cmul(u_G, s_5)), cmul(u_Gc, cmul(p_T4, u_z))), cmul(p_T4, cmul(p_dc4, u_z))), cmul(p_T4, cmul(p_Tc4, cmul(u_z, u_zc))));
  small_solve(5, A, b, s);
  q[0] = s[0];
  q[1] = s[1];
  q[2] = s[2];
  q[3] = s[3];
  q[4] = s[4];
}

static const or_plugin OR_PLUGINS[] = {
  {1, "conic2", 2, 12, plug_conic2_rows, plug_conic2_start},
  {2, "burmester5", 5, 20, plug_burmester5_rows, plug_burmester5_start},
};
#define OR_NUM_PLUGINS 2
