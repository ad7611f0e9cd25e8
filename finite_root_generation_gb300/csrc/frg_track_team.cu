// Warp-cooperative path-tracking kernels: one 8-lane team per path, 4 paths per
// warp, the linear algebra register-resident (frg_team.cuh) and the path state in
// shared memory.
//
// The control flow is the reference's TrackPath (htpytrack.cu:33-220) with
// DormandPrince65 (rungekutta.cu:3-123) and Newton (htpysupport.cu:407-494),
// restated as the same state machine as the one-thread-per-path kernel
// (frg_track.cu), with identical decisions, tolerances, counters and random draws.
// Every trip of the loop runs one warp-convergent linear step for all four teams
// (the expensive part), then each team's control transitions with team-masked
// shuffles; vector updates are spread over the team's lanes (element e on lane e % 8).
//
// Modes as in frg_track.cu: MODE_PLAIN (FP64 from start to root), MODE_LO (FP32
// stage; every path is handed to the FP64 kernel, either to continue or, when it
// ended on a step limit, just to be finished), MODE_RESUME (FP64 continuation and
// finishing of handed-off paths).
#include <cuda_runtime.h>
#include <stdint.h>

#include "frg_kernels.h"
#include "frg_team.cuh"

namespace frg {
namespace team {

enum Phase : int { PH_FETCH = 0, PH_TANGENT0 = 1, PH_RK = 2, PH_NEWTON = 3, PH_SHARP = 4, PH_IDLE = 5 };
enum Mode : int { MODE_PLAIN = 0, MODE_LO = 1, MODE_RESUME = 2 };

// Draw index of start-value component m (frgkinematics.cu:41-58 order): one draw per
// uniform value, two per complex-normal component.
__device__ __forceinline__ double start_component(uint64_t seed, uint64_t stream, int m, int dist, double range) {
  if (dist == 0) return 2.0 * range * frg_uniform01(seed, stream, (uint64_t)m) - range;
  const double u1 = frg_uniform01(seed, stream, 2ull * m), u2 = frg_uniform01(seed, stream, 2ull * m + 1);
  return sqrt(-log(u1)) * cospi(2.0 * u2);
}

// GenerateStart (frgkinematics.cu:13-136) spread over the team: every lane draws
// the 14 link values and P0, Pc0; lane g solves the two quadratics of its own j
// (lane 7 repeats j = 7). Outputs: links z[0..13], U_j, and the lane's parameters
// P0, Pc0, Pj, Pcj, Qj, Qcj (all FP64).
__device__ void team_start(uint64_t seed, uint64_t stream, int dist, double range, int j, cd* z, cd& Uj,
                           cd* sp) {
#pragma unroll 1
  for (int i = 0; i < 14; ++i)
    z[i] = cd(start_component(seed, stream, 2 * i, dist, range), start_component(seed, stream, 2 * i + 1, dist, range));
  const cd P0(start_component(seed, stream, 28, dist, range), start_component(seed, stream, 29, dist, range));
  const cd Pc0(start_component(seed, stream, 30, dist, range), start_component(seed, stream, 31, dist, range));
  const cd Rj(start_component(seed, stream, 32 + 2 * (j - 1), dist, range),
              start_component(seed, stream, 33 + 2 * (j - 1), dist, range));
  const uint64_t pmbase = (dist == 0 ? 46ull : 92ull) + 2ull * (j - 1);
  const cd A = z[0], B = z[1], C = z[2], D = z[3], F = z[4], G = z[5], H = z[6];
  const cd Ac = z[7], Bc = z[8], Cc = z[9], Dc = z[10], Fc = z[11], Gc = z[12], Hc = z[13];
  const cd iR = cinv(Rj);
  cd Aq = (G - D) * (iR * (Hc - Gc) - (Hc - Fc));
  cd Acq = (Gc - Dc) * (Rj * (H - G) - (H - F));
  cd Bq = (-(Rj * ((H - G) * (Hc - Fc))) - iR * ((Hc - Gc) * (H - F))) +
          ((G - D) * (Gc - Dc) + ((H - G) * (Hc - Gc) + ((H - F) * (Hc - Fc) - (F - D) * (Fc - Dc))));
  double pm = frg_uniform01(seed, stream, pmbase) < 0.5 ? -1.0 : 1.0;
  cd disc = csqrt_halfangle(Bq * Bq - 4.0 * (Aq * Acq));
  const cd TUc = cinv(2.0 * Aq) * (-Bq + pm * disc);
  const cd SUc = cinv(F - D) * (TUc * (G - D) + (Rj * (H - G) - (H - F)));
  const cd w = (Rj * (H - C) - SUc * (F - B)) - (H - F);
  const cd wc = (iR * (Hc - Cc) - cinv(SUc) * (Fc - Bc)) - (Hc - Fc);
  Aq = (Ac - Bc) * w;
  Acq = (A - B) * wc;
  Bq = w * wc + ((A - B) * (Ac - Bc) - (C - A) * (Cc - Ac));
  pm = frg_uniform01(seed, stream, pmbase + 1) < 0.5 ? -1.0 : 1.0;
  disc = csqrt_halfangle(Bq * Bq - 4.0 * (Aq * Acq));
  Uj = cinv(2.0 * Aq) * (-Bq + pm * disc);
  const cd QUc = cdiv(cd(-1.0), C - A) * (cinv(Uj) * (A - B) + w);
  const cd Qj = QUc * Uj;
  const cd S = SUc * Uj;
  sp[0] = P0;
  sp[1] = Pc0;
  sp[2] = B + (S * (F - B) + Uj * (P0 - F));
  sp[3] = Bc + (cinv(S) * (Fc - Bc) + cinv(Uj) * (Pc0 - Fc));
  sp[4] = Qj;
  sp[5] = cinv(Qj);
}

template <typename T> __device__ __forceinline__ const cx<T>* fpm_of(const TrackArgs& a, int task);
template <> __device__ __forceinline__ const cx<double>* fpm_of<double>(const TrackArgs& a, int task) {
  return a.fpm + (size_t)task * NP;
}
template <> __device__ __forceinline__ const cx<float>* fpm_of<float>(const TrackArgs& a, int task) {
  return a.fpm_lo + (size_t)task * NP;
}
// the task's parameters and gamma in the point type (FP64, or double-float)
template <typename P> __device__ __forceinline__ const cx<P>* fpm_hi_of(const TrackArgs& a, int task);
template <> __device__ __forceinline__ const cx<double>* fpm_hi_of<double>(const TrackArgs& a, int task) {
  return a.fpm + (size_t)task * NP;
}
template <> __device__ __forceinline__ const cx<df>* fpm_hi_of<df>(const TrackArgs& a, int task) {
  return a.fpm_df + (size_t)task * NP;
}
template <typename P> __device__ __forceinline__ cx<P> gamma_hi_of(const TrackArgs& a, int task);
template <> __device__ __forceinline__ cx<double> gamma_hi_of<double>(const TrackArgs& a, int task) {
  return a.gamma[task];
}
template <> __device__ __forceinline__ cx<df> gamma_hi_of<df>(const TrackArgs& a, int task) {
  return a.gamma_df[task];
}
template <typename T> __device__ __forceinline__ cx<T> gamma_of(const TrackArgs& a, int task);
template <> __device__ __forceinline__ cx<double> gamma_of<double>(const TrackArgs& a, int task) {
  return a.gamma[task];
}
template <> __device__ __forceinline__ cx<float> gamma_of<float>(const TrackArgs& a, int task) {
  return a.gamma_lo[task];
}

// Finish a path (FP64, spread over the team): finite check, dehomogenize
// (frg.cu:44-46, :60), canonical cognate (frgkinematics.cu:227-285, frg.cu:63-65), the
// row-scaled residual of the target system at the root, outputs and counters. id is the
// path's global index, ti its task-set index.
__device__ void team_finish(const TrackArgs& a, Smem<double>& S, const cd* Yf, int64_t id, int ti, int code,
                            int g, unsigned tmask, int n_ivp, int n_newton, int steps) {
  const cd* fpm = a.fpm + (size_t)ti * NP;
  if (a.yfinal)
    for (int e = g; e < NY; e += TEAM) a.yfinal[(size_t)id * NY + e] = Yf[e];
  double zl = 0.0;
  for (int e = g; e < NV; e += TEAM) zl = fmax(zl, sqrt(cnorm2(Yf[e])));
  const double zmax = team_max(tmask, zl);
  const cd z0 = Yf[NV];
  if (code == 0 && a.cfg.inf_tol > 0.0 && sqrt(cnorm2(z0)) < a.cfg.inf_tol * zmax) code = FRG_CODE_INFINITE;
  // dehomogenized point into S.Ye (SwitchPatch with u = e_21: scale 1/Z0)
  const cd iz = cdiv(cd(1.0), z0);
  __syncwarp(tmask);
  for (int e = g; e < NV; e += TEAM) S.Ye[e] = iz * Yf[e];
  __syncwarp(tmask);
  // 1/2 cognate into S.dx: U_down by lane g for j = g + 1, the link sides by lane 0
  if (g < 7) {
    const int i = g + 1;
    const cd B = S.Ye[1], F = S.Ye[4];
    S.dx[13 + i] = ((fpm[i] - B) - S.Ye[13 + i] * (fpm[0] - F)) * cinv(F - B);
  }
  if (g == 0) {
    cognate12(S.Ye, fpm[0], S.dx);
    cognate12(S.Ye + 7, fpm[8], S.dx + 7);
  }
  __syncwarp(tmask);
  const bool swap = S.dx[0].re < S.Ye[0].re;
  cd root_e[3];
  int ne = 0;
  for (int e = g; e < NV; e += TEAM) {
    const cd r = swap ? S.dx[e] : S.Ye[e];
    a.roots[(size_t)id * NV + e] = r;
    root_e[ne++] = r;
  }
  __syncwarp(tmask);
  for (int e = g, m = 0; e < NV; e += TEAM, ++m) S.Ye[e] = root_e[m];
  __syncwarp(tmask);
  if (a.resid) {
    // lane g evaluates group j = g + 1 at [root, 1] with q = fpm, dq = 0
    const int j = g < 7 ? g + 1 : 7;
    const cd one(1.0), zero(0.0);
    FrgGroupOut<double> o;
    const cd* R = S.Ye;
    frg_group_eval<double>(R[0], R[1], R[2], R[3], R[4], R[5], R[6], R[7], R[8], R[9], R[10], R[11], R[12], R[13],
                           one, cinv(R[4] - R[1]), cinv(R[6] - R[2]), cinv(R[11] - R[8]), cinv(R[13] - R[9]), one,
                           one, fpm[0], fpm[8], zero, zero, R[13 + j], cinv(R[13 + j]), fpm[j], fpm[8 + j],
                           fpm[15 + j], fpm[22 + j], zero, zero, zero, zero, o);
    double m0 = 0.0, m1 = 0.0, m2 = 0.0;
    for (int c = 0; c < 8; ++c) m0 = fmax(m0, fmax(fabs(o.dI[c].re), fabs(o.dI[c].im)));
    for (int c = 0; c < 6; ++c) m1 = fmax(m1, fmax(fabs(o.dII[c].re), fabs(o.dII[c].im)));
    for (int c = 0; c < 16; ++c) m2 = fmax(m2, fmax(fabs(o.dIII[c].re), fabs(o.dIII[c].im)));
    const double r0 = sqrt(cnorm2(o.fI)) / m0, r1 = sqrt(cnorm2(o.fII)) / m1, r2 = sqrt(cnorm2(o.fIII)) / m2;
    // fmax drops NaN operands: a non-finite row makes the residual infinite instead
    double r = (r0 == r0 && r1 == r1 && r2 == r2) ? fmax(r0, fmax(r1, r2)) : INFINITY;
    r = team_max(tmask, r);
    if (g == 0) a.resid[id] = r;
  }
  if (g == 0) {
    a.codes[id] = code;
    if (a.work) {
      a.work[(size_t)id * 3 + 0] = n_ivp;
      a.work[(size_t)id * 3 + 1] = n_newton;
      a.work[(size_t)id * 3 + 2] = steps;
    }
    if (a.counters) {
      atomicAdd(&a.counters[code & 7], 1ull);
      atomicAdd(&a.counters[8], (unsigned long long)n_ivp);
      atomicAdd(&a.counters[9], (unsigned long long)n_newton);
      atomicAdd(&a.counters[10], (unsigned long long)steps);
    }
  }
  __syncwarp(tmask);
}

// Tracking features of a path at a checkpoint (an accepted step), the early-retirement
// network's input: progress in t, step sizes now and at the last two checkpoints,
// condition estimates, the homogenizer's share |Z0| / max|Z| (which goes to 0 on
// paths diverging to infinity), step and rejection counts, patch switches and the
// corrector's behaviour. One lane computes them from the shared state.
template <typename P>
__device__ void path_features(const cx<P>* Yc, double s, double rmax, int step, int ministep, uint64_t rng_index,
                              double ck_t1, double ck_t2, double ck_s1, double ck_s2, bool fp64, int n_ivp,
                              int n_newton, double residual, int streak, int tstepQ, int bounces, float* x) {
  double zmax = 0.0;
  for (int e = 0; e < 21; ++e) {
    const cd v = cd(Yc[e]);
    zmax = fmax(zmax, sqrt(cnorm2(v)));
  }
  const double z0 = sqrt(cnorm2(cd(Yc[21])));
  const double t = double(Yc[22].re);
  const auto lg = [](double v) { return (float)log10(fmax(v, 1e-30)); };
  for (int k = 0; k < FRG_MLP_IN; ++k) x[k] = 0.f;
  x[0] = (float)t;
  x[1] = lg(fmax(1.0 - t, 1e-16));
  x[2] = lg(s);
  x[3] = lg(fmax(rmax, 1.0));
  x[4] = lg(z0 / fmax(zmax, 1e-300));
  x[5] = lg(zmax);
  x[6] = step * 1e-3f;
  x[7] = ministep * 1e-3f;
  x[8] = (float)(ministep - 2 * step) / (float)(ministep > 0 ? ministep : 1);
  x[9] = (float)((double)(rng_index > 92 ? rng_index - 92 : 0) / 46.0 * 0.1);
  x[10] = (float)(t - ck_t1);
  x[11] = lg(fmax(t - ck_t1, 1e-16));
  x[12] = (float)(ck_t1 - ck_t2);
  x[13] = lg(ck_s1 > 0 ? ck_s1 : s);
  x[14] = lg(ck_s2 > 0 ? ck_s2 : s);
  x[15] = fp64 ? 1.f : 0.f;
  x[16] = (float)n_newton / (float)(n_ivp > 0 ? n_ivp : 1);
  x[17] = lg(residual);
  x[18] = streak * 0.1f;
  x[19] = (float)tstepQ;
  x[20] = bounces * 0.125f;
  for (int k = 0; k < FRG_MLP_IN; ++k)  // non-finite inputs (an infinite condition estimate, a NaN residual)
    x[k] = (x[k] - x[k] == 0.f) ? fminf(fmaxf(x[k], -100.f), 100.f) : 100.f;
}

// One lane's work at a checkpoint: record the features and/or score them with the
// network; returns 1 to retire the path. Not inlined, so its arrays stay off the
// tracking loop's registers.
template <typename P>
__device__ __noinline__ int checkpoint(const TrackArgs& a, const cx<P>* Yc, int64_t id, double s, double rmax,
                                       int step, int ministep, uint64_t rng_index, double ck_t1, double ck_t2,
                                       double ck_s1, double ck_s2, bool fp64, int n_ivp, int n_newton,
                                       double residual, int streak, int tstepQ, int bounces) {
  float x[FRG_MLP_IN];
  path_features<P>(Yc, s, rmax, step, ministep, rng_index, ck_t1, ck_t2, ck_s1, ck_s2, fp64, n_ivp, n_newton,
                   residual, streak, tstepQ, bounces, x);
  if (a.feat && a.nfeat) {
    const int k = a.nfeat[id];
    if (k < a.feat_max) {
      float* dst = a.feat + ((size_t)id * a.feat_max + k) * FRG_MLP_IN;
      for (int f = 0; f < FRG_MLP_IN; ++f) dst[f] = x[f];
      a.nfeat[id] = k + 1;
    }
  }
  if (!a.mlp.w) return 0;
  for (int f = 0; f < FRG_MLP_IN; ++f) x[f] = (x[f] - a.mlp.mu[f]) * a.mlp.inv_sigma[f];
  float z[FRG_MLP_OUT];
  mlp_logits(a.mlp.w, x, z);
  const int retire = mlp_prob(z, 1) >= a.mlp.threshold;
  if (retire && a.counters) atomicAdd(&a.counters[36], 1ull);
  return retire;
}

template <int MODE, typename T, typename P = typename PointOf<T>::type>
__global__ void __launch_bounds__(FRG_TEAM_THREADS) team_kernel(TrackArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool LO = (MODE == MODE_LO);
  const unsigned FULL = 0xffffffffu;
  const frg_config& c = a.cfg;
  const int lane = threadIdx.x & 31;
  const int g = lane & 7;
  const unsigned tmask = 0xffu << (lane & 24);
  typedef cx<P> cp;
  Smem<T, P>& S = reinterpret_cast<Smem<T, P>*>(smem_raw)[threadIdx.x >> 3];
  {
    cx<T>* base = reinterpret_cast<cx<T>*>(&S);
    for (int i = g; i < (int)(sizeof(Smem<T, P>) / sizeof(cx<T>)); i += TEAM) base[i] = cx<T>(T(0));
  }
  // The FP32 stage's corrector iterates on FP32 residuals until |dY| falls below
  // newt_tol_lo (or stops shrinking), then on FP64 residuals to the reference's
  // newt_tol: an FP32 LU with FP64 residuals converges like FP64 Newton while the
  // pivot ratio stays below cond_switch.
  const T newt_tol = T(c.newt_tol);
  const int jg = g < 7 ? g + 1 : 7;
  // what this launch works through: fresh paths, paths resumed in FP32 (lo_list),
  // or paths handed to FP64 (handoff_list)
  const bool lo_resume = LO && a.lo_list != nullptr && !a.carry;
  const int64_t ncarry = (LO && a.carry && a.lo_list != nullptr) ? (int64_t)*a.lo_count : 0;
  const int64_t nqueue = (MODE == MODE_RESUME) ? (int64_t)*a.handoff_count
                         : (lo_resume ? (int64_t)*a.lo_count : ncarry + a.npaths);
  // A path returns from FP64 to the next round's FP32 kernel after handback_good
  // consecutive well-conditioned solves, or after fp64_segment FP64 solves in this launch
  // (FP64 latency per solve is high on this part, so long FP64 segments set a launch's
  // tail; a path still ill conditioned is simply handed over again by the FP32 kernel).
  const int kBackSteps = c.handback_good > 0 ? c.handback_good : 0x7fffffff;
  const int kSegment = c.fp64_segment > 0 ? c.fp64_segment : 96;
  constexpr int kMaxBounces = 64;

  LaneParams<T> lp;
  int64_t id = -1;      // global path index: records, lists, outputs
  int64_t lid = 0;      // index within the path's round: random stream, start values, task
  int ti = 0;           // task-set index (round * ntasks + task): parameters, gamma
  uint64_t pseed = a.seed;
  T s = T(0), err = T(0), scale = T(0), residual = T(100);
  int tstepQ = 0, streak = 0, step = 0, ministep = 0, stage = 0, attempt = 0, it = 0, code = 0;
  int n_ivp = 0, n_newton = 0;
  uint64_t rng_index = 0;
  int phase = PH_FETCH;
  bool hires = !LO;
  T res_prev = T(0);
  int good = 0, bounces = 0, seg = 0;
  // checkpoints of the early-retirement network (history kept in S.ck_*)
  const bool checkpoints = a.feat_every > 0 && (a.feat != nullptr || a.mlp.w != nullptr);
  unsigned long long fp64_solves = 0;
  // cycle accounting (lane 0 of each warp): fetch, setup, linear step, transitions;
  // warp steps and active-team steps
  long long cyc[4] = {0, 0, 0, 0};
  long long warp_steps = 0, team_steps = 0, refine_steps = 0, refine_warp = 0, res_cyc = 0;
  __syncwarp();

  for (;;) {
    long long tc0 = clock64();
    // =========================================================== fetch (per team)
    while (phase == PH_FETCH) {
      unsigned long long qi = 0;
      if (g == 0) qi = atomicAdd(a.queue, 1ull);
      qi = __shfl_sync(tmask, qi, 0, TEAM);
      if ((int64_t)qi >= nqueue) { phase = PH_IDLE; break; }
      const bool carried = (int64_t)qi < ncarry;
      id = (MODE == MODE_RESUME) ? a.handoff_list[qi]
           : (lo_resume || carried) ? a.lo_list[qi] : a.round_base + ((int64_t)qi - ncarry);
      const bool resumed = MODE == MODE_RESUME || lo_resume || carried;
      const int64_t round = id / a.npaths;
      lid = id - round * a.npaths;
      pseed = a.seeds ? a.seeds[round] : a.seed;
      int lo = 0, hi = a.ntasks - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.task_start[mid] <= lid) lo = mid; else hi = mid - 1;
      }
      ti = (int)(round * a.ntasks) + lo;
      {
        cd z[14], Uj, sp[6];
        // start values precomputed by the start kernel hold this launch's round only; a
        // path of an earlier round (carried over) regenerates them (the same code, the
        // same values)
        if (a.starts && round * a.npaths == a.round_base) {
          const cd* st = a.starts + (size_t)lid * FRG_START_STRIDE;
          for (int e = g; e < 14; e += TEAM) z[e] = st[e];
          Uj = st[13 + jg];
#pragma unroll
          for (int i = 0; i < 6; ++i) sp[i] = st[21 + param_index(i, jg)];
        } else {
          team_start(pseed, (uint64_t)(lid + c.path_offset), c.start_dist, c.start_range, jg, z, Uj, sp);
        }
        const cx<T>* fpmT = fpm_of<T>(a, ti);
#pragma unroll
        for (int i = 0; i < 6; ++i) { lp.sp[i] = cx<T>(sp[i]); lp.fp[i] = fpmT[param_index(i, jg)]; }
        lp.gamma = gamma_of<T>(a, ti);
        if (g < 7) {
          S.spm[jg] = cp(sp[2]); S.spm[8 + jg] = cp(sp[3]); S.spm[15 + jg] = cp(sp[4]); S.spm[22 + jg] = cp(sp[5]);
        }
        if (g == 0) { S.spm[0] = cp(sp[0]); S.spm[8] = cp(sp[1]); }
        if (!resumed) {
          for (int e = g; e < 14; e += TEAM) S.Yc[e] = cp(z[e]);
          if (g < 7) S.Yc[13 + jg] = cp(Uj);
          if (g == 7) { S.Yc[21] = cp(P(1)); S.Yc[22] = cp(P(0)); }
        }
      }
      code = 0; stage = 0; attempt = 0; it = 0; residual = T(100); err = T(0); scale = T(0);
      good = 0; bounces = 0; seg = 0;
      if (g == 0) { S.ck_t[0] = S.ck_t[1] = 0.0; S.ck_s[0] = S.ck_s[1] = 0.f; S.ck_rmax = 0.f; }
      if (resumed) {
        const Handoff& h = a.handoff[id];
        for (int e = g; e < NY; e += TEAM) {
          S.Yc[e] = cp(h.Yc[e]); S.Vc[e] = cx<T>(h.Vc[e]); S.u[e] = cx<T>(h.u[e]);
        }
        s = T(h.s); rng_index = h.rng_index; streak = h.streak; step = h.step; ministep = h.ministep;
        tstepQ = h.tstepQ; n_ivp = h.n_ivp; n_newton = h.n_newton; bounces = h.bounces;
        __syncwarp(tmask);
        if (h.reason == 6) {  // the path already ended on a step limit in the FP32 stage
          if constexpr (!LO) {
            cd Yf[NY];
            for (int e = 0; e < NY; ++e) Yf[e] = h.Yc[e];
            team_finish(a, *reinterpret_cast<Smem<double>*>(&S), Yf, id, ti, h.code, g, tmask, n_ivp, n_newton,
                        step);
          }
          continue;  // next path
        }
        phase = PH_RK;
      } else {
        __syncwarp(tmask);
        // TrackPath's patches start at draw 0 of the path's stream (by-value state,
        // frg.cu:54,57); u (htpytrack.cu:53-58) then the random velocity patch (:63-67).
        const double R = c.patch_range;
        const uint64_t stream = (uint64_t)(lid + c.path_offset);
        for (int e = g; e < NY; e += TEAM) {
          S.u[e] = cx<T>(T(2.0 * R * frg_uniform01(pseed, stream, 2 * e) - R),
                         T(2.0 * R * frg_uniform01(pseed, stream, 2 * e + 1) - R));
          S.Vc[e] = cx<T>(T(2.0 * R * frg_uniform01(pseed, stream, 46 + 2 * e) - R),
                          T(2.0 * R * frg_uniform01(pseed, stream, 47 + 2 * e) - R));
        }
        rng_index = 92;
        __syncwarp(tmask);
        // SwitchPatch(u, Yc, Yc) (htpytrack.cu:60), in the point type
        cp d(P(0));
        for (int e = g; e < NZ; e += TEAM) d = cfma(cp(S.u[e]), S.Yc[e], d);
        d = cp(team_sum(tmask, d.re), team_sum(tmask, d.im));
        const cp sc = cdiv(cp(P(1)) - cp(S.u[22]) * S.Yc[22], d);
        __syncwarp(tmask);
        for (int e = g; e < NZ; e += TEAM) S.Yc[e] = sc * S.Yc[e];
        s = T(c.s_init); tstepQ = 0; streak = c.caution_steps - 1; step = 0; ministep = 0;
        n_ivp = 0; n_newton = 0;
        phase = PH_TANGENT0;
      }
    }
    if (__all_sync(FULL, phase == PH_IDLE)) break;
    long long tc1 = clock64();

    // ==================================================== set up (per team)
    const bool newton = (phase == PH_NEWTON || phase == PH_SHARP);
    bool tstep = false;
    T tgoal = T(0);
    const cx<T>* Wsrc = S.Vc;
    cx<T>* dst = S.dx;
    if (phase == PH_TANGENT0 || phase == PH_IDLE) {
      for (int e = g; e < NY; e += TEAM) S.Ye[e] = cx<T>(S.Yc[e]);
    } else if (phase == PH_RK) {
      tstep = tstepQ != 0;
      dst = S.k[stage];
      if (stage == 0) {
        for (int e = g; e < NY; e += TEAM) S.Ye[e] = cx<T>(S.Yc[e]);
      } else {
        Wsrc = S.k[stage - 1];
        const double* w = c_dpA[stage];
        for (int e = g; e < NY; e += TEAM) {
          cx<T> acc = T(w[stage - 1]) * s * S.k[stage - 1][e];
          for (int l = stage - 2; l >= 0; --l) acc = T(w[l]) * s * S.k[l][e] + acc;
          S.Ye[e] = cx<T>(S.Yc[e]) + acc;
        }
      }
    } else {
      tgoal = (phase == PH_SHARP) ? T(1) : T(S.Yn[22].re);
      for (int e = g; e < NY; e += TEAM) S.Ye[e] = cx<T>(S.YN[e]);
    }
    __syncwarp();
    long long tc2 = clock64();

    // ========================================== linear step (whole warp)
    const StepOut<T> r = linear_step<T, P>(S, Wsrc, dst, newton, tstep, tgoal, lp, fpm_hi_of<P>(a, ti),
                                        gamma_hi_of<P>(a, ti), g, hires);
    __syncwarp();
    long long tc3 = clock64();
    if (lane == 0) {
      cyc[0] += tc1 - tc0; cyc[1] += tc2 - tc1; cyc[2] += tc3 - tc2;
      warp_steps++;
      res_cyc += r.res_cycles;
    }
    {
      const unsigned act = __ballot_sync(FULL, phase != PH_IDLE && g == 0);
      if (lane == 0) team_steps += __popc(act);
      if (LO) {  // corrector iterations on double-float residuals, and warp steps that ran one
        const unsigned ref = __ballot_sync(FULL, phase != PH_IDLE && g == 0 && newton && hires);
        if (lane == 0) { refine_steps += __popc(ref); refine_warp += ref != 0u; }
      }
    }
    if (phase == PH_IDLE) continue;
    if (!LO) ++fp64_solves;
    if (checkpoints && g == 0) S.ck_rmax = fmaxf(S.ck_rmax, (float)r.ratio);
    if (MODE == MODE_RESUME) {
      good = (r.ratio < T(c.cond_switch * 1e-2)) ? good + 1 : 0;
      ++seg;
    }
    if (newton) ++n_newton; else ++n_ivp;

    // ============================================= transitions (per team)
    bool finished = false;
    int handoff = 0;
    bool handback = false;
    bool final_from_YN = false;
    if (LO && !(r.ratio <= T(c.cond_switch)) && !(a.lo_keep_ill && r.ratio - r.ratio == T(0))) {
      handoff = 2;  // ill-conditioned (or non-finite) step: continue in FP64 from Yc
    } else if (MODE == MODE_RESUME && c.fp64_budget > 0 && seg >= c.fp64_budget) {
      code = 2;  // the FP64 budget of this path is spent: retire it as a step-limit failure
      finished = true;
    } else if (phase == PH_TANGENT0) {
      for (int e = g; e < NY; e += TEAM) S.Vc[e] = S.dx[e];
      if (c.max_steps == 0) { code = 1; finished = true; }
      stage = 0;
      phase = PH_RK;
    } else if (phase == PH_RK) {
      if (++stage == 8) {
        stage = 0;
        // error estimate and step factor (rungekutta.cu:99-112), prediction (:115-122)
        T es = T(0);
        for (int e = g; e < NY; e += TEAM) {
          cx<T> le = T(c_dpE[7]) * s * S.k[7][e];
          cx<T> yb = T(c_dpB[7]) * s * S.k[7][e];
          for (int l = 6; l >= 0; --l) {
            if (c_dpE[l] != 0.0) le = T(c_dpE[l]) * s * S.k[l][e] + le;
            if (c_dpB[l] != 0.0) yb = T(c_dpB[l]) * s * S.k[l][e] + yb;
          }
          es += cnorm2(le);
          S.Yn[e] = S.Yc[e] + cp(yb);
          S.Vn[e] = S.k[7][e];
        }
        err = sqrt(team_sum(tmask, es));
        scale = (err > T(10e-17)) ? T(0.8) * pow(T(c.rk_tol) / err, T(1) / T(6)) : T(5);
        if (scale > T(5)) scale = T(5);
        __syncwarp(tmask);
        if (ministep++ == c.max_ministeps) { code = 2; finished = true; }
        else if (err <= T(c.rk_tol)) {
          const double tn = double(S.Yn[22].re);
          if (LO && !c.lo_endgame && tn > 1.0 - c.nudge_trigger) handoff = 5;  // the endgame runs in FP64
          else if (tn <= 1.0 - c.nudge_trigger) { attempt = 0; phase = PH_NEWTON; }
          else if (fabs(1.0 - tn) < c.sharp_trigger) { attempt = 0; phase = PH_SHARP; }
          else { tstepQ = 1; s = T(1.0 - double(S.Yc[22].re)); }  // land on t = 1 (htpytrack.cu:120-123)
          if (phase == PH_NEWTON || phase == PH_SHARP) {
            for (int e = g; e < NY; e += TEAM) S.YN[e] = S.Yn[e];
            // the FP32 stage sharpens at exactly t = 1 (its t-update is only FP32-accurate)
            if (LO && phase == PH_SHARP && g == (22 & 7)) S.YN[22] = cp(P(1));
            residual = T(100);
            it = 0;
            hires = !LO || phase == PH_SHARP;
          }
        } else if (s <= T(c.s_min)) {
          if (LO) handoff = 4; else { code = 3; finished = true; }
        } else {
          s *= scale;
          if (s < T(c.s_min)) s = T(c.s_min * 0.9);
          streak = 0;
        }
      }
    } else {
      // one corrector or sharpening iteration (htpysupport.cu:427-492)
      const bool sharp = (phase == PH_SHARP);
      const int max_its = sharp ? c.sharp_its : c.newt_its;
      const T tol = sharp ? T(c.sharp_tol) : newt_tol;
      const int restype = (LO || sharp) ? (LO ? 1 : c.sharp_residual) : c.newt_residual;
      bool done = false, predicted = false;
      if (restype == 0 && it > 0) {
        residual = r.hnorm;  // |H| at the current point: the residual of the previous update
        if (!(it < max_its && residual > tol)) done = true;
      }
      if (!done) {
        for (int e = g; e < NY; e += TEAM) S.YN[e] += cp(S.dx[e]);
        it++;
        if (restype != 0) {
          residual = sqrt(r.xnorm2);
          if (LO && !hires) {
            // FP32 residuals: at the FP32 noise floor either accept (no refinement) or
            // continue on double-float residuals to the reference's tolerance
            const bool conv = residual < T(c.newt_tol_lo);
            const bool floor_ = conv || (it > 1 && residual > T(0.5) * res_prev);
            if (c.lo_refine == 3 && conv && !sharp) {
              // the FP32 update is already below newt_tol_lo: accept it without refining
              done = true;
              predicted = true;
            } else {
              if (floor_ && c.lo_refine) hires = true;
              if ((floor_ && !c.lo_refine) || !(it < max_its)) done = true;
            }
          } else if (!(it < max_its && residual > tol)) {
            done = true;
          } else if (LO && !sharp && c.lo_refine == 2 &&
                     residual * (r.ratio * T(1e-6) + residual * T(100)) < T(0.1) * tol) {
            // refined iteration whose successor is predicted below the tolerance: the
            // FP32 solve contracts the error by about cond * 2^-24 (ratio * 1e-6 with a
            // safety factor of 16) on top of Newton's quadratic term
            done = true;
            predicted = true;
          }
          res_prev = residual;
        }
      }
      __syncwarp(tmask);
      if (done) {
        const bool ok = predicted || ((LO && !c.lo_refine && !sharp)
                                          ? residual < T(c.newt_tol_lo) * T(100)
                                          : (hires || !LO) && residual < (sharp ? T(c.sharp_tol) : newt_tol));
        if (ministep++ == c.max_ministeps) { code = 2; finished = true; final_from_YN = sharp; }
        else if (ok && !sharp) {
          if (fabs(1.0 - double(S.Yn[22].re)) < c.sharp_trigger) {
            if (LO && !c.lo_endgame) handoff = 5;
            attempt = 0; phase = PH_SHARP;
            for (int e = g; e < NY; e += TEAM) S.YN[e] = S.Yn[e];
            if (LO && g == (22 & 7)) S.YN[22] = cp(P(1));
            residual = T(100); it = 0; hires = true;
          } else {
            // accept the step (htpytrack.cu:176-183)
            for (int e = g; e < NY; e += TEAM) { S.Yc[e] = S.YN[e]; S.Vc[e] = S.Vn[e]; }
            streak++;
            if (streak < c.caution_steps && scale > T(1)) scale = T(1);
            s *= scale;
            if (s > T(c.s_max)) s = T(c.s_max);
            else if (s < T(c.s_min)) s = T(c.s_min * 0.9);
            step++;
            if (checkpoints && step % a.feat_every == 0) {
              // checkpoint: record the features and/or let the network retire the path
              int retire = 0;
              __syncwarp(tmask);
              if (g == 0)
                retire = checkpoint<P>(a, S.Yc, id, double(s), S.ck_rmax, step, ministep, rng_index, S.ck_t[0],
                                       S.ck_t[1], S.ck_s[0], S.ck_s[1], !LO, n_ivp, n_newton, double(residual),
                                       streak, tstepQ, bounces);
              retire = __shfl_sync(tmask, retire, 0, TEAM);
              if (g == 0) {
                S.ck_t[1] = S.ck_t[0]; S.ck_t[0] = double(S.Yc[22].re);
                S.ck_s[1] = S.ck_s[0]; S.ck_s[0] = float(s); S.ck_rmax = 0.f;
              }
              if (retire) { code = 2; finished = true; }  // retired early: reported as a step-limit failure
            }
            if (finished) {
            } else if (step == c.max_steps) { code = 1; finished = true; }
            else if (LO && !c.lo_endgame && double(S.YN[22].re) >= c.t_switch) handoff = 1;
            else if (MODE == MODE_RESUME && a.back_list && (good >= kBackSteps || seg >= kSegment) &&
                     bounces < kMaxBounces && (c.lo_endgame || double(S.YN[22].re) < c.t_switch))
              handback = true;  // back to FP32 (well conditioned again, or the segment is used up)
            else { stage = 0; phase = PH_RK; }
          }
        } else if (ok && sharp) {
          code = 0; finished = true; final_from_YN = true;
        } else {
          // new random patch and SwitchPatch(u, Yn, Yn) (htpytrack.cu:145-151, :204-210)
          const double R = c.patch_range;
          const uint64_t stream = (uint64_t)(lid + c.path_offset);
          for (int e = g; e < NY; e += TEAM)
            S.u[e] = cx<T>(T(2.0 * R * frg_uniform01(pseed, stream, rng_index + 2 * e) - R),
                           T(2.0 * R * frg_uniform01(pseed, stream, rng_index + 2 * e + 1) - R));
          rng_index += 46;
          __syncwarp(tmask);
          cp d(P(0));
          for (int e = g; e < NZ; e += TEAM) d = cfma(cp(S.u[e]), S.Yn[e], d);
          d = cp(team_sum(tmask, d.re), team_sum(tmask, d.im));
          const cp sc = cdiv(cp(P(1)) - cp(S.u[22]) * S.Yn[22], d);
          __syncwarp(tmask);
          for (int e = g; e < NZ; e += TEAM) S.Yn[e] = sc * S.Yn[e];
          if (!sharp) {
            if (++attempt < c.newt_attempts) {
              for (int e = g; e < NY; e += TEAM) S.YN[e] = S.Yn[e];
              residual = T(100); it = 0; hires = !LO;
            } else if (s <= T(c.s_min)) {
              if (LO) handoff = 3; else { code = 4; finished = true; }
            } else {
              s *= T(0.5);
              if (s < T(c.s_min)) s = T(c.s_min * 0.9);
              streak = 0;
              stage = 0;
              phase = PH_RK;
            }
          } else {
            if (++attempt < c.sharp_attempts) {
              for (int e = g; e < NY; e += TEAM) S.YN[e] = S.Yn[e];
              if (LO && g == (22 & 7)) S.YN[22] = cp(P(1));
              residual = T(100); it = 0;
            } else if (LO) {
              handoff = 5;  // the FP32 stage could not sharpen: the FP64 kernel retries the endgame
            } else {
              code = 5; finished = true; final_from_YN = true;
            }
          }
        }
      }
    }
    __syncwarp(tmask);
    if (lane == 0) cyc[3] += clock64() - tc3;

    if (MODE == MODE_RESUME && (finished || handback) && g == 0 && a.counters) {
      // length of this path's FP64 segment in this launch
      const int b = seg < 100 ? 0 : seg < 300 ? 1 : seg < 1000 ? 2 : seg < 3000 ? 3 : seg < 10000 ? 4 : 5;
      atomicAdd(&a.counters[40 + b], 1ull);
      atomicMax(&a.counters[46], (unsigned long long)seg);
    }
    if ((LO && (handoff || finished)) || handback) {
      // save the state for the other precision's kernel (an FP32 path is always
      // finished in FP64; an FP64 path well conditioned again returns to FP32)
      Handoff& h = a.handoff[id];
      const cp* ysrc = (finished && final_from_YN) ? S.YN : S.Yc;  // a sharpened root is in YN
      for (int e = g; e < NY; e += TEAM) { h.Yc[e] = cd(ysrc[e]); h.Vc[e] = cd(S.Vc[e]); h.u[e] = cd(S.u[e]); }
      if (g == 0) {
        h.s = double(s); h.rng_index = rng_index; h.streak = streak; h.step = step; h.ministep = ministep;
        h.tstepQ = tstepQ; h.n_ivp = n_ivp; h.n_newton = n_newton;
        h.reason = finished ? 6 : handoff; h.code = code;
        h.bounces = bounces + (handback ? 1 : 0);
        if (a.counters) {
          if (handback) atomicAdd(&a.counters[13], 1ull);
          else {
            if (!finished) atomicAdd(&a.counters[12], 1ull);
            atomicAdd(&a.counters[15 + (finished ? 6 : handoff)], 1ull);
          }
        }
        unsigned long long* cnt = handback ? a.back_count : a.handoff_count;
        int64_t* list = handback ? a.back_list : a.handoff_list;
        const unsigned long long slot = atomicAdd(cnt, 1ull);
        list[slot] = id;
      }
      __syncwarp(tmask);
      phase = PH_FETCH;
      continue;
    }
    if (finished) {
      if constexpr (!LO) {
        cd Yf[NY];
        const cp* src = final_from_YN ? S.YN : S.Yc;
        for (int e = 0; e < NY; ++e) Yf[e] = cd(src[e]);
        __syncwarp(tmask);
        team_finish(a, S, Yf, id, ti, code, g, tmask, n_ivp, n_newton, step);
      }
      phase = PH_FETCH;
    }
  }
  if (a.counters && fp64_solves && g == 0) atomicAdd(&a.counters[11], fp64_solves);
  if (a.counters && lane == 0) {
    const int base = LO ? 24 : 30;
    for (int i = 0; i < 4; ++i) atomicAdd(&a.counters[base + i], (unsigned long long)cyc[i]);
    atomicAdd(&a.counters[base + 4], (unsigned long long)warp_steps);
    atomicAdd(&a.counters[base + 5], (unsigned long long)team_steps);
    if (LO) {
      atomicAdd(&a.counters[22], (unsigned long long)refine_steps);
      atomicAdd(&a.counters[23], (unsigned long long)refine_warp);
      atomicAdd(&a.counters[37], (unsigned long long)res_cyc);
    }
  }
}

}  // namespace team
}  // namespace frg

namespace frg {
namespace team {
// GenerateStart per path, one team per path (the same lane split as the tracking
// kernels' inline generation, so the values are identical).
__global__ void __launch_bounds__(FRG_TEAM_THREADS) start_kernel(TrackArgs a, cd* starts) {
  const int g = threadIdx.x & 7;
  const int64_t id = ((int64_t)blockIdx.x * FRG_TEAM_THREADS + threadIdx.x) >> 3;
  if (id >= a.npaths) return;
  const int jg = g < 7 ? g + 1 : 7;
  cd z[14], Uj, sp[6];
  team_start(a.seed, (uint64_t)(id + a.cfg.path_offset), a.cfg.start_dist, a.cfg.start_range, jg, z, Uj, sp);
  cd* st = starts + (size_t)id * FRG_START_STRIDE;
  for (int e = g; e < 14; e += TEAM) st[e] = z[e];
  if (g < 7) {
    st[13 + jg] = Uj;
    st[21 + jg] = sp[2]; st[21 + 8 + jg] = sp[3]; st[21 + 15 + jg] = sp[4]; st[21 + 22 + jg] = sp[5];
  }
  if (g == 0) { st[21] = sp[0]; st[21 + 8] = sp[1]; }
}
}  // namespace team
}  // namespace frg

cudaError_t frg_launch_starts(const frg::TrackArgs& args, cx<double>* starts, cudaStream_t stream) {
  const int64_t blocks = (args.npaths * 8 + FRG_TEAM_THREADS - 1) / FRG_TEAM_THREADS;
  frg::team::start_kernel<<<(unsigned)blocks, FRG_TEAM_THREADS, 0, stream>>>(args, starts);
  return cudaGetLastError();
}

namespace {
template <int MODE, typename T, typename P = typename frg::team::PointOf<T>::type>
cudaError_t team_launch(const frg::TrackArgs& args, int grid, cudaStream_t stream) {
  const size_t smem = (FRG_TEAM_THREADS / 8) * sizeof(frg::team::Smem<T, P>);
  cudaError_t e = cudaFuncSetAttribute(frg::team::team_kernel<MODE, T, P>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  frg::team::team_kernel<MODE, T, P><<<grid, FRG_TEAM_THREADS, smem, stream>>>(args);
  return cudaGetLastError();
}
template <int MODE, typename T, typename P = typename frg::team::PointOf<T>::type>
cudaError_t team_occ(int* bps) {
  const size_t smem = (FRG_TEAM_THREADS / 8) * sizeof(frg::team::Smem<T, P>);
  cudaError_t e = cudaFuncSetAttribute(frg::team::team_kernel<MODE, T, P>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, frg::team::team_kernel<MODE, T, P>, FRG_TEAM_THREADS,
                                                       smem);
}
}  // namespace

cudaError_t frg_launch_team(int mode, const frg::TrackArgs& args, int grid, cudaStream_t stream) {
  switch (mode) {
    case 0: return team_launch<frg::team::MODE_PLAIN, double>(args, grid, stream);
    case 1: return team_launch<frg::team::MODE_LO, float>(args, grid, stream);
    case 2: return team_launch<frg::team::MODE_RESUME, double>(args, grid, stream);
    case 3: return team_launch<frg::team::MODE_LO, float, df>(args, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t frg_team_occupancy(int mode, int* blocks_per_sm) {
  switch (mode) {
    case 0: return team_occ<frg::team::MODE_PLAIN, double>(blocks_per_sm);
    case 1: return team_occ<frg::team::MODE_LO, float>(blocks_per_sm);
    case 2: return team_occ<frg::team::MODE_RESUME, double>(blocks_per_sm);
    case 3: return team_occ<frg::team::MODE_LO, float, df>(blocks_per_sm);
    default: return cudaErrorInvalidValue;
  }
}
