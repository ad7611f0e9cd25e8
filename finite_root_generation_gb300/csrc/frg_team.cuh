// Team (8-lane) building blocks of the warp-cooperative tracker.
//
// A team of 8 consecutive lanes tracks one path; a warp holds 4 teams. Lane g < 7
// owns equation group j = g + 1 (rows j-1, j+6, j+13 of the reference's JH,
// htpysupport.cu:89-144); lane 7 owns the two patch rows (the projective patch u,
// row 21, and the velocity patch / t-selector, row 22).
//
// The linear system of one step (the reference's 23x23 row-scaled dense LU,
// LinearSolve / LinearSolveNewton, htpysupport.cu:146-400) is solved with the
// system's structure: U_j appears only in group j's three equations and in the two
// patch rows, so each group lane pivots U_j out of its own rows (partial pivoting
// among the group's three rows) and the eliminations are folded into the patch rows
// with one butterfly reduction. What remains is a dense 16 x 16 system in the links
// A..Hc, the homogenizer Z0 and t, two rows per lane, solved by LU with partial
// pivoting across the team (argmax and pivot-row broadcast by warp shuffles), then
// column-oriented back substitution; U_j follows from lane g's pivot row. The
// solution is the same as the dense solve up to rounding (checked against the
// dense LU in the tests).
//
// Register-resident: a lane holds at most 3 rows of 18 complex values during the
// group phase and 2 rows of 17 during the dense phase. The Newton variant replaces
// the velocity patch by the t-selector row with right-hand side t_goal - t, which
// fixes dt exactly like LinearSolveNewton's x[22] = tdiff (htpysupport.cu:374).
#pragma once

#include "frg_device.cuh"

namespace frg {
namespace team {

constexpr int TEAM = 8;
constexpr int NG = 16;  // links (14), Z0, t
constexpr int VS = 24;  // shared-memory vector stride (23 used)

// reduced-system column -> state index
__device__ __forceinline__ constexpr int gstate(int c) { return c < 14 ? c : (c == 14 ? 21 : 22); }

template <typename T>
__device__ __forceinline__ T shfl(unsigned mask, T v, int src) { return __shfl_sync(mask, v, src, TEAM); }
template <typename T>
__device__ __forceinline__ T shfl_xor(unsigned mask, T v, int off) { return __shfl_xor_sync(mask, v, off, TEAM); }
template <typename T>
__device__ __forceinline__ cx<T> shfl(unsigned mask, cx<T> v, int src) {
  return cx<T>(__shfl_sync(mask, v.re, src, TEAM), __shfl_sync(mask, v.im, src, TEAM));
}
template <typename T>
__device__ __forceinline__ cx<T> shfl_xor(unsigned mask, cx<T> v, int off) {
  return cx<T>(__shfl_xor_sync(mask, v.re, off, TEAM), __shfl_xor_sync(mask, v.im, off, TEAM));
}
template <typename T>
__device__ __forceinline__ T team_sum(unsigned mask, T v) {
  v += shfl_xor(mask, v, 4);
  v += shfl_xor(mask, v, 2);
  v += shfl_xor(mask, v, 1);
  return v;
}
template <typename T>
__device__ __forceinline__ T team_max(unsigned mask, T v) {
  v = fmax(v, shfl_xor(mask, v, 4));
  v = fmax(v, shfl_xor(mask, v, 2));
  v = fmax(v, shfl_xor(mask, v, 1));
  return v;
}
template <typename T>
__device__ __forceinline__ T team_min(unsigned mask, T v) {
  v = fmin(v, shfl_xor(mask, v, 4));
  v = fmin(v, shfl_xor(mask, v, 2));
  v = fmin(v, shfl_xor(mask, v, 1));
  return v;
}

// Per-team shared state of one path, in the working precision. The 32-byte pad
// makes the stride between teams 32 bytes past a multiple of 128, so the four teams
// of a warp reading "the same" field hit four different bank groups.
template <typename T>
struct Smem {
  cx<T> Yc[VS], Vc[VS], Yn[VS], Vn[VS], YN[VS], u[VS], Ye[VS], dx[VS];
  cx<T> k[8][VS];
  unsigned char pad[32];
};

// Parameter values a lane needs for its group: index 0 P0, 1 Pc0, 2 Pj, 3 Pcj, 4 Qj, 5 Qcj.
template <typename T>
struct LaneParams {
  cx<T> sp[6], fp[6];
  cx<T> gamma;
};

__device__ __forceinline__ int param_index(int slot, int j) {
  switch (slot) {
    case 0: return 0;
    case 1: return 8;
    case 2: return j;
    case 3: return 8 + j;
    case 4: return 15 + j;
    default: return 22 + j;
  }
}

template <typename T>
struct StepOut {
  T ratio;   // pivot ratio max|u_ii| / min|u_ii| over all 23 pivots
  T xnorm2;  // |x|^2 of the (normalised, for tangents) solution
  T hnorm;   // |H| at the evaluation point (Newton)
};

// One linear-system step, executed convergently by the whole warp (full-mask
// shuffles inside). Each team evaluates at its S.Ye:
//   tangent (newton = false): [JH; W] x = e_23 with W = the velocity patch Wsrc,
//     then normalised to unit length with real dt/ds (or dt = 1 when tstep),
//     Im(dt) = 0 (htpysupport.cu:237-299);
//   Newton (newton = true): [JH; e_t] x = [-H; tgoal - t] (htpysupport.cu:427-477).
// The solution is written to dst[0..22] (shared memory).
template <typename T>
__device__ __forceinline__ StepOut<T> linear_step(Smem<T>& S, const cx<T>* Wsrc, cx<T>* dst, bool newton,
                                                  bool tstep, T tgoal, const LaneParams<T>& lp, int g) {
  const unsigned FULL = 0xffffffffu;
  const bool grp = g < 7;
  const int j = grp ? g + 1 : 7;
  const cx<T> zero(T(0));

  // ---- evaluation point and parameters q(t), dq/dt (htpysupport.cu:37-62)
  const cx<T> A = S.Ye[0], B = S.Ye[1], C = S.Ye[2], D = S.Ye[3], F = S.Ye[4], G = S.Ye[5], H = S.Ye[6];
  const cx<T> Ac = S.Ye[7], Bc = S.Ye[8], Cc = S.Ye[9], Dc = S.Ye[10], Fc = S.Ye[11], Gc = S.Ye[12],
              Hc = S.Ye[13];
  const cx<T> z = S.Ye[21];
  const T t = S.Ye[22].re;
  const cx<T> U = S.Ye[13 + j];
  cx<T> q[6], dq[6];
  {
    const cx<T> g1t = lp.gamma * (T(1) - t);
    const cx<T> iden = cinv(g1t + cx<T>(t));
    const cx<T> gid2 = lp.gamma * (iden * iden);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      q[i] = (g1t * lp.sp[i] + t * lp.fp[i]) * iden;
      dq[i] = (lp.fp[i] - lp.sp[i]) * gid2;
    }
  }
  // ---- the group's equations, derivatives and t-column (generated code)
  FrgGroupOut<T> o;
  {
    const cx<T> z2 = z * z, z3 = z2 * z;
    frg_group_eval<T>(A, B, C, D, F, G, H, Ac, Bc, Cc, Dc, Fc, Gc, Hc, z, cinv(F - B), cinv(H - C),
                      cinv(Fc - Bc), cinv(Hc - Cc), z2, z3, q[0], q[1], dq[0], dq[1], U, cinv(U), q[2], q[3],
                      q[4], q[5], dq[2], dq[3], dq[4], dq[5], o);
  }
  // rows in local column order: 0..13 links, 14 Z0, 15 t, 16 U_j, 17 rhs
  cx<T> r0[18], r1[18], r2[18];
#pragma unroll
  for (int c = 0; c < 18; ++c) { r0[c] = zero; r1[c] = zero; r2[c] = zero; }
  r0[0] = o.dI[0]; r0[2] = o.dI[1]; r0[6] = o.dI[2]; r0[7] = o.dI[3]; r0[9] = o.dI[4]; r0[13] = o.dI[5];
  r0[16] = o.dI[6]; r0[14] = o.dI[7]; r0[15] = o.tI;
  r1[1] = o.dII[0]; r1[4] = o.dII[1]; r1[8] = o.dII[2]; r1[11] = o.dII[3];
  r1[16] = o.dII[4]; r1[14] = o.dII[5]; r1[15] = o.tII;
#pragma unroll
  for (int c = 0; c < 14; ++c) r2[c] = o.dIII[c];
  r2[16] = o.dIII[14]; r2[14] = o.dIII[15]; r2[15] = o.tIII;
  if (newton) { r0[17] = -o.fI; r1[17] = -o.fII; r2[17] = -o.fIII; }
  T hsq = grp ? cnorm2(o.fI) + cnorm2(o.fII) + cnorm2(o.fIII) : T(0);
  // row scaling by 1/max(|re|,|im|) (htpysupport.cu:259-277, :446-471)
  {
    T m0 = T(0), m1 = T(0), m2 = T(0);
#pragma unroll
    for (int c = 0; c < 17; ++c) {
      m0 = fmax(m0, fmax(tabs(r0[c].re), tabs(r0[c].im)));
      m1 = fmax(m1, fmax(tabs(r1[c].re), tabs(r1[c].im)));
      m2 = fmax(m2, fmax(tabs(r2[c].re), tabs(r2[c].im)));
    }
    const T s0 = T(1) / m0, s1 = T(1) / m1, s2 = T(1) / m2;
#pragma unroll
    for (int c = 0; c < 18; ++c) { r0[c] = s0 * r0[c]; r1[c] = s1 * r1[c]; r2[c] = s2 * r2[c]; }
  }
  // ---- eliminate U_j inside the group: partial pivoting among its three rows
  const T a0 = cnorm2(r0[16]), a1 = cnorm2(r1[16]), a2 = cnorm2(r2[16]);
  const int p = (a0 >= a1 && a0 >= a2) ? 0 : (a1 >= a2 ? 1 : 2);
  cx<T> piv[18], ra[17], rb[17];
#pragma unroll
  for (int c = 0; c < 18; ++c) piv[c] = p == 0 ? r0[c] : (p == 1 ? r1[c] : r2[c]);
  cx<T> ipu = cinv(piv[16]);
  {
    const cx<T> la = (p == 0 ? r1[16] : r0[16]) * ipu;
    const cx<T> lb = (p == 2 ? r1[16] : r2[16]) * ipu;
#pragma unroll
    for (int c = 0; c < 17; ++c) {
      const int cc = c < 16 ? c : 17;
      const cx<T> xa = p == 0 ? r1[cc] : r0[cc];
      const cx<T> xb = p == 2 ? r1[cc] : r2[cc];
      ra[c] = cfms(xa, la, piv[cc]);
      rb[c] = cfms(xb, lb, piv[cc]);
    }
  }
  // ---- patch rows (lane 7) and the folding of every group's pivot row into them
  const cx<T>* u = S.u;
  T su = T(0);
#pragma unroll
  for (int e = 0; e < 23; ++e) su = fmax(su, fmax(tabs(u[e].re), tabs(u[e].im)));
  su = T(1) / su;
  const T tdiff = tgoal - t;
  cx<T> hu(T(0));
  if (newton) {
#pragma unroll
    for (int e = 0; e < 23; ++e) hu = cfma(u[e], S.Ye[e], hu);
    hu = hu - cx<T>(T(1));
  }
  if (!grp) { hsq = cnorm2(hu); ipu = zero; }
  const cx<T> mu = (su * u[13 + j]) * ipu;
  const cx<T> mw = newton ? zero : Wsrc[13 + j] * ipu;
  cx<T> Su[17], Sw[17];
#pragma unroll
  for (int c = 0; c < 17; ++c) {
    const cx<T> pc = piv[c < 16 ? c : 17];
    Su[c] = mu * pc;
    Sw[c] = mw * pc;
  }
#pragma unroll
  for (int c = 0; c < 17; ++c) {
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1) {
      Su[c] += shfl_xor(FULL, Su[c], off);
      Sw[c] += shfl_xor(FULL, Sw[c], off);
    }
  }
  cx<T> R0[17], R1[17];
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const cx<T> uc = su * u[gstate(c)];
    const cx<T> wc = newton ? (c == 15 ? cx<T>(T(1)) : zero) : Wsrc[gstate(c)];
    R0[c] = grp ? ra[c] : uc - Su[c];
    R1[c] = grp ? rb[c] : wc - Sw[c];
  }
  R0[16] = grp ? ra[16] : (newton ? -(su * hu) : zero) - Su[16];
  R1[16] = grp ? rb[16] : (newton ? cx<T>(tdiff) : cx<T>(T(1))) - Sw[16];

  // ---- dense 16 x 16 LU with partial pivoting across the team
  int step0 = 99, step1 = 99;  // elimination step at which each row became a pivot
  cx<T> ipiv[16];
  int powner[16];
  T pmax = T(0), pmin = T(3.0e38);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const T v0 = step0 < 99 ? T(-1) : cnorm2(R0[k]);
    const T v1 = step1 < 99 ? T(-1) : cnorm2(R1[k]);
    T bv = v0 >= v1 ? v0 : v1;
    int bk = 2 * g + (v0 >= v1 ? 0 : 1);
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1) {
      const T ov = shfl_xor(FULL, bv, off);
      const int ok = shfl_xor(FULL, bk, off);
      if (ov > bv || (ov == bv && ok < bk)) { bv = ov; bk = ok; }
    }
    const int pl = bk >> 1, ps = bk & 1;
    powner[k] = bk;
    if (g == pl) { if (ps) step1 = k; else step0 = k; }
    cx<T> prow[17];
#pragma unroll
    for (int c = k; c < 17; ++c) prow[c] = shfl(FULL, ps ? R1[c] : R0[c], pl);
    const cx<T> ip = cinv(prow[k]);
    ipiv[k] = ip;
    const T pa = sqrt(cnorm2(prow[k]));
    pmax = fmax(pmax, pa);
    pmin = fmin(pmin, pa);
    const cx<T> l0 = step0 < 99 ? zero : R0[k] * ip;
    const cx<T> l1 = step1 < 99 ? zero : R1[k] * ip;
#pragma unroll
    for (int c = k + 1; c < 17; ++c) {
      R0[c] = cfms(R0[c], l0, prow[c]);
      R1[c] = cfms(R1[c], l1, prow[c]);
    }
  }
  // ---- back substitution, column by column
  cx<T> xg[16];
#pragma unroll
  for (int k = 15; k >= 0; --k) {
    const int pl = powner[k] >> 1, ps = powner[k] & 1;
    const cx<T> mine = (ps ? R1[16] : R0[16]) * ipiv[k];
    const cx<T> xk = shfl(FULL, mine, pl);
    xg[k] = xk;
    const cx<T> m0 = step0 < k ? R0[k] : zero;
    const cx<T> m1 = step1 < k ? R1[k] : zero;
    R0[16] = cfms(R0[16], m0, xk);
    R1[16] = cfms(R1[16], m1, xk);
  }
  // ---- U_j from the group's pivot row
  cx<T> xu = piv[17];
#pragma unroll
  for (int c = 0; c < 16; ++c) xu = cfms(xu, piv[c], xg[c]);
  xu = xu * ipu;
  // ---- pivot ratio over all 23 pivots
  {
    const T gp = grp ? sqrt(cnorm2(piv[16])) : pmax;
    pmax = fmax(pmax, team_max(FULL, gp));
    pmin = fmin(pmin, team_min(FULL, grp ? gp : pmin));
  }
  // ---- normalisation and output
  T n2 = T(0);
#pragma unroll
  for (int c = 0; c < 16; ++c) n2 += cnorm2(xg[c]);
  n2 += team_sum(FULL, grp ? cnorm2(xu) : T(0));
  StepOut<T> out;
  out.hnorm = sqrt(team_sum(FULL, hsq));
  out.ratio = pmax / pmin;
  if (!newton) {
    const cx<T> xt = xg[15];
    cx<T> sc;
    if (!tstep) sc = cx<T>(xt.re, -xt.im) * (T(1) / (sqrt(cnorm2(xt)) * sqrt(n2)));
    else sc = cinv(xt);
#pragma unroll
    for (int c = 0; c < 16; ++c) xg[c] = sc * xg[c];
    xu = sc * xu;
    xg[15].im = T(0);
    n2 = n2 * cnorm2(sc);
  }
  out.xnorm2 = n2;
  if (grp) dst[13 + j] = xu;
#pragma unroll
  for (int c = 0; c < 16; ++c)
    if ((c & 7) == g) dst[gstate(c)] = xg[c];
  return out;
}

}  // namespace team
}  // namespace frg
