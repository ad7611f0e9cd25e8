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
#include "frg_df.cuh"

namespace frg {
namespace team {

// Type of the path's points (Yc, Yn, YN) and of the FP32 stage's refinement residual:
// FP64 by default; the FP32 stage can instead keep them in double-float (P = df), which
// runs on the FP32 pipes but is ~10x more code than the FP64 form.
template <typename T> struct PointOf { typedef double type; };

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
__device__ __forceinline__ df shfl_xor(unsigned mask, df v, int off) {
  return df(__shfl_xor_sync(mask, v.hi, off, TEAM), __shfl_xor_sync(mask, v.lo, off, TEAM));
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

// Per-team shared state of one path. The points Yc (accepted), Yn (predicted) and
// YN (corrector iterate) are in the point type (FP64, or double-float in the FP32
// stage, whose corrector refines on double-float residuals with an FP32 solve);
// directions, patches and stage vectors are in the working precision T. U/Urhs hold the reduced system's
// upper factor for the back substitution. The 32-byte tail makes the stride between
// teams 32 bytes past a multiple of 128, so the four teams of a warp reading "the
// same" field hit different bank groups.
template <typename T, typename P = typename PointOf<T>::type>
struct Smem {
  cx<P> Yc[VS], Yn[VS], YN[VS];
  cx<P> spm[32];
  cx<T> Vc[VS], Vn[VS], u[VS], Ye[VS], dx[VS];
  cx<T> k[8][VS];
  cx<T> U[16][16];
  cx<T> Urhs[16];
  // Checkpoint history of the early-retirement features (lane 0 only). These 32 bytes
  // also make the stride between teams 32 bytes past a multiple of 128.
  double ck_t[2];   // t at the last two checkpoints
  float ck_s[2];    // step sizes at the last two checkpoints
  float ck_rmax;    // largest condition estimate since the last checkpoint
  float ck_unused;
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
  T ratio;   // condition estimate (pivot ratios of the elimination), +inf if not finite
  T xnorm2;  // |x|^2 of the (normalised, for tangents) solution
  T hnorm;   // |H| at the evaluation point (Newton)
  long long res_cycles;  // cycles the warp spent in the refinement residual (FP32 stage)
};

// The team's residual F_j (its three equations) at the point Yd with q(t), all in
// the point type P (htpysupport.cu:37-48, :64-86): the FP32 stage's corrector uses it
// as the right-hand side, so its iterates converge in double-float although J and
// the LU are FP32.
template <typename P>
__device__ __forceinline__ void residual_hi(const cx<P>* Yd, const cx<P>* spm, const cx<P>* fpm, cx<P> gamma,
                                            int j, cx<P>& fI, cx<P>& fII, cx<P>& fIII) {
  typedef cx<P> cp;
  const P t = Yd[22].re;
  const cp g1t = gamma * (P(1) - t);
  const cp iden = cinv(g1t + cp(t));
  cp q[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int pi = param_index(i, j);
    q[i] = (g1t * spm[pi] + t * fpm[pi]) * iden;
  }
  const cp z = Yd[21], z2 = z * z, z3 = z2 * z, U = Yd[13 + j];
  frg_group_f<P>(Yd[0], Yd[1], Yd[2], Yd[3], Yd[4], Yd[5], Yd[6], Yd[7], Yd[8], Yd[9], Yd[10], Yd[11],
                      Yd[12], Yd[13], z, cinv(Yd[4] - Yd[1]), cinv(Yd[6] - Yd[2]), cinv(Yd[11] - Yd[8]),
                      cinv(Yd[13] - Yd[9]), z2, z3, q[0], q[1], U, cinv(U), q[2], q[3], q[4], q[5], fI, fII, fIII);
}

// One step of the dense phase over a window of W columns: the current pivot column
// is index 0; rows shift one column left as they are eliminated, so a rolled loop
// needs no dynamic register indexing. The pivot row (final once chosen) goes to S.U.
template <typename T, int W, typename P>
__device__ __forceinline__ void lu_window_step(Smem<T, P>& S, int k, int g, cx<T>* R0, cx<T>& R0r, cx<T>* R1,
                                               cx<T>& R1r, bool& used0, bool& used1, T& pmax, T& pmin) {
  const unsigned FULL = 0xffffffffu;
  const cx<T> zero(T(0));
  const T v0 = used0 ? T(-1) : cnorm2(R0[0]);
  const T v1 = used1 ? T(-1) : cnorm2(R1[0]);
  T bv = v0 >= v1 ? v0 : v1;
  int bk = 2 * g + (v0 >= v1 ? 0 : 1);
#pragma unroll
  for (int off = 4; off >= 1; off >>= 1) {
    const T ov = shfl_xor(FULL, bv, off);
    const int ok = shfl_xor(FULL, bk, off);
    if (ov > bv || (ov == bv && ok < bk)) { bv = ov; bk = ok; }
  }
  const int pl = bk >> 1, ps = bk & 1;
  if (g == pl) { if (ps) used1 = true; else used0 = true; }
  cx<T> prow[W];
#pragma unroll
  for (int c = 0; c < W; ++c) prow[c] = shfl(FULL, ps ? R1[c] : R0[c], pl);
  const cx<T> prhs = shfl(FULL, ps ? R1r : R0r, pl);
  const cx<T> ip = cinv(prow[0]);
  if (g == 0) {  // the diagonal keeps the pivot's reciprocal for the back substitution
    S.U[k][k] = ip;
#pragma unroll
    for (int c = 1; c < W; ++c)
      if (k + c < 16) S.U[k][k + c] = prow[c];
    S.Urhs[k] = prhs;
  }
  const T pa = cnorm2(prow[0]);  // squared pivot magnitude
  pmax = fmax(pmax, pa);
  pmin = fmin(pmin, pa);
  const cx<T> l0 = used0 ? zero : R0[0] * ip;
  const cx<T> l1 = used1 ? zero : R1[0] * ip;
#pragma unroll
  for (int c = 0; c + 1 < W; ++c) {
    R0[c] = cfms(R0[c + 1], l0, prow[c + 1]);
    R1[c] = cfms(R1[c + 1], l1, prow[c + 1]);
  }
  R0[W - 1] = zero;
  R1[W - 1] = zero;
  R0r = cfms(R0r, l0, prhs);
  R1r = cfms(R1r, l1, prhs);
}

// One linear-system step, executed convergently by the whole warp (full-mask
// shuffles inside). Each team evaluates at its S.Ye:
//   tangent (newton = false): [JH; W] x = e_23 with W = the velocity patch Wsrc,
//     then normalised to unit length with real dt/ds (or dt = 1 when tstep),
//     Im(dt) = 0 (htpysupport.cu:237-299);
//   Newton (newton = true): [JH; e_t] x = [-H; tgoal - t] (htpysupport.cu:427-477),
//     H at the FP64 point S.YN; when T is float, H is evaluated in FP64 if `hires`
//     and in FP32 (at the rounded point) otherwise.
// The solution is written to dst[0..22] (shared memory).
template <typename T, typename P>
__device__ __forceinline__ StepOut<T> linear_step(Smem<T, P>& S, const cx<T>* Wsrc, cx<T>* dst, bool newton,
                                                  bool tstep, T tgoal, const LaneParams<T>& lp,
                                                  const cx<P>* fpm_hi, cx<P> gamma_hi, int g, bool hires) {
  const unsigned FULL = 0xffffffffu;
  const bool grp = g < 7;
  const int j = grp ? g + 1 : 7;
  const cx<T> zero(T(0));
  constexpr bool LOWP = sizeof(T) < sizeof(P);
  // `newton` and `hires` are per team, so reductions inside branches on them use the
  // team's own mask; everything outside such branches runs on the full warp
  const unsigned tmask = 0xffu << (threadIdx.x & 24);

  // ---- FP64 residual of the corrector (FP32 stage only)
  cx<T> hF0 = zero, hF1 = zero, hF2 = zero, hU = zero;
  T hsq = T(0);
  long long res_cycles = 0;
  const long long t_res0 = LOWP ? clock64() : 0;
  if (LOWP && newton && hires) {
    cx<P> fI, fII, fIII;
    residual_hi<P>(S.YN, S.spm, fpm_hi, gamma_hi, j, fI, fII, fIII);
    // patch residual u . YN - 1, its 23 terms spread over the team
    cx<P> d(P(0));
    for (int e = g; e < 23; e += TEAM) d = cfma(cx<P>(S.u[e]), S.YN[e], d);
    d = cx<P>(team_sum(tmask, d.re), team_sum(tmask, d.im)) - cx<P>(P(1));
    hF0 = cx<T>(fI); hF1 = cx<T>(fII); hF2 = cx<T>(fIII); hU = cx<T>(d);
    hsq = grp ? T(cnorm2(hF0) + cnorm2(hF1) + cnorm2(hF2)) : T(cnorm2(hU));
  }
  if (LOWP) res_cycles = clock64() - t_res0;

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
  const bool lores_h = !LOWP || !hires;  // H from the working-precision evaluation
  if (lores_h) {
    hF0 = o.fI; hF1 = o.fII; hF2 = o.fIII;
    hsq = grp ? cnorm2(o.fI) + cnorm2(o.fII) + cnorm2(o.fIII) : T(0);
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
  if (newton) { r0[17] = -hF0; r1[17] = -hF1; r2[17] = -hF2; }
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
  cx<T> piv[18], R0[16], R1[16], R0r, R1r;
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
      const cx<T> ya = cfms(xa, la, piv[cc]);
      const cx<T> yb = cfms(xb, lb, piv[cc]);
      if (c < 16) { R0[c] = ya; R1[c] = yb; } else { R0r = ya; R1r = yb; }
    }
  }
  // ---- patch rows (lane 7) and the folding of every group's pivot row into them
  const cx<T>* u = S.u;
  T su = T(0);
  for (int e = g; e < 23; e += TEAM) su = fmax(su, fmax(tabs(u[e].re), tabs(u[e].im)));
  su = T(1) / team_max(FULL, su);
  const T tdiff = tgoal - t;
  if (lores_h && newton) {  // patch residual u . Ye - 1, its 23 terms spread over the team
    cx<T> d(T(0));
    for (int e = g; e < 23; e += TEAM) d = cfma(u[e], S.Ye[e], d);
    hU = cx<T>(team_sum(tmask, d.re), team_sum(tmask, d.im)) - cx<T>(T(1));
  }
  if (!grp) {
    if (lores_h) hsq = cnorm2(hU);
    ipu = zero;
  }
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
  if (!grp) {
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      R0[c] = su * u[gstate(c)] - Su[c];
      R1[c] = (newton ? (c == 15 ? cx<T>(T(1)) : zero) : Wsrc[gstate(c)]) - Sw[c];
    }
    R0r = (newton ? -(su * hU) : zero) - Su[16];
    R1r = (newton ? cx<T>(tdiff) : cx<T>(T(1))) - Sw[16];
  }

  // ---- re-scale the 16 dense rows (max(|re|,|im|) = 1): eliminating U_j can shrink a
  //      group row by cancellation, and unequal rows would mislead both the pivot
  //      choice and the pivot-ratio condition estimate (with the re-scaling the ratio
  //      tracks the reference's 23 x 23 row-scaled elimination)
  {
    T m0 = T(0), m1 = T(0);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      m0 = fmax(m0, fmax(tabs(R0[c].re), tabs(R0[c].im)));
      m1 = fmax(m1, fmax(tabs(R1[c].re), tabs(R1[c].im)));
    }
    const T s0 = T(1) / m0, s1 = T(1) / m1;
#pragma unroll
    for (int c = 0; c < 16; ++c) { R0[c] = s0 * R0[c]; R1[c] = s1 * R1[c]; }
    R0r = s0 * R0r;
    R1r = s1 * R1r;
  }
  // ---- dense 16 x 16 LU with partial pivoting across the team: 8 steps over a
  //      16-wide window, then 8 over the remaining 8 columns
  bool used0 = false, used1 = false;
  T pmax = T(0), pmin = T(3.0e38);
#pragma unroll 1
  for (int k = 0; k < 8; ++k) lu_window_step<T, 16, P>(S, k, g, R0, R0r, R1, R1r, used0, used1, pmax, pmin);
  {
    cx<T> Q0[8], Q1[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) { Q0[c] = R0[c]; Q1[c] = R1[c]; }
#pragma unroll 1
    for (int k = 8; k < 16; ++k) lu_window_step<T, 8, P>(S, k, g, Q0, R0r, Q1, R1r, used0, used1, pmax, pmin);
  }
  __syncwarp();
  // ---- back substitution, column by column; lane g keeps the right-hand sides of
  //      pivot rows g and g + 8
  cx<T> rb0 = S.Urhs[g], rb1 = S.Urhs[g + 8];
  __syncwarp();
#pragma unroll 1
  for (int k = 15; k >= 0; --k) {
    const cx<T> mine = ((k >> 3) ? rb1 : rb0) * S.U[k][k];
    const cx<T> xk = shfl(FULL, mine, k & 7);
    if (g == 0) S.Urhs[k] = xk;
    if (g < k) rb0 = cfms(rb0, S.U[g][k], xk);
    if (g + 8 < k) rb1 = cfms(rb1, S.U[g + 8][k], xk);
  }
  __syncwarp();
  cx<T> xg[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) xg[c] = S.Urhs[c];
  // ---- U_j from the group's pivot row
  cx<T> xu = piv[17];
#pragma unroll
  for (int c = 0; c < 16; ++c) xu = cfms(xu, piv[c], xg[c]);
  xu = xu * ipu;
  // ---- condition estimate: the larger of the dense phase's pivot ratio and the
  //      worst group amplification 1/|u_jj| (a group's pivot row is row-scaled, so its
  //      largest entry is about 1, and U_j's error grows like eps / |u_jj|). A
  //      non-finite solution (zero or non-finite pivot) makes it infinite.
  T ratio;
  {
    const T ig = grp ? T(1) / cnorm2(piv[16]) : T(0);
    ratio = sqrt(fmax(pmax / pmin, team_max(FULL, ig)));
  }
  // ---- normalisation and output
  T n2 = T(0);
#pragma unroll
  for (int c = 0; c < 16; ++c) n2 += cnorm2(xg[c]);
  n2 += team_sum(FULL, grp ? cnorm2(xu) : T(0));
  StepOut<T> out;
  out.res_cycles = res_cycles;
  out.hnorm = sqrt(team_sum(FULL, hsq));
  out.ratio = (n2 - n2 == T(0)) ? ratio : T(INFINITY);  // n2 - n2 is NaN iff n2 is not finite
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
  __syncwarp();
  if (grp) dst[13 + j] = xu;
#pragma unroll
  for (int c = 0; c < 16; ++c)
    if ((c & 7) == g) dst[gstate(c)] = xg[c];
  return out;
}

}  // namespace team
}  // namespace frg
