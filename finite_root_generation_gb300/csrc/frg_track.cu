// The path-tracking kernels.
//
// One CUDA thread tracks one path at a time and pulls the next path index from a
// device work queue (an atomic counter) when its path ends, so the very uneven
// path lengths (tens to thousands of steps) do not hold a whole launch back the
// way the reference's one-path-per-thread launch does (frg.cu:25-27, :374).
//
// The reference's nested tracking loops (TrackPath, htpytrack.cu:83-216, with
// DormandPrince65, rungekutta.cu:3-123, and Newton, htpysupport.cu:407-494) are
// restated as a state machine in which every trip performs exactly one linear
// system step -- Jacobian evaluation, row scaling, LU and solve, either a
// predictor tangent (IVP, htpysupport.cu:237-299) or a corrector iteration -- so
// the expensive part runs converged across the warp while the cheap control logic
// around it diverges. The decisions, tolerances, counters and random draws are the
// reference's, so a path ends with the reference's code and root.
//
// Three modes, each instantiated for Stephenson II (SysStephenson2) and for every
// generated plug-in system (frg_plugins_gen.cuh), whose sizes set the path state and
// the dense system:
//   MODE_PLAIN   FP64 throughout, from the start system to the root (the reference's
//                arithmetic);
//   MODE_LO      FP32 state and linear algebra from the start system; a path is handed
//                to FP64 (its state saved to HBM) when t reaches t_switch, when an LU
//                pivot ratio exceeds cond_switch, when a prediction enters the endgame
//                (t > 1 - nudge_trigger), or when a step would fail at s_min;
//   MODE_RESUME  FP64, continuing handed-off paths from their saved state through the
//                endgame and sharpening.
#include <cuda_runtime.h>
#include <stdint.h>

#include "frg_device.cuh"
#include "frg_kernels.h"
#include "frg_plugins_gen.cuh"

namespace frg {

enum Phase : int { PH_FETCH = 0, PH_TANGENT0 = 1, PH_RK = 2, PH_NEWTON = 3, PH_SHARP = 4 };
enum Mode : int { MODE_PLAIN = 0, MODE_LO = 1, MODE_RESUME = 2 };

// NY_ = the path state's length (homogeneous unknowns + t), NP_ = parameters.
template <typename T, int NY_, int NP_>
struct PathState {
  cx<T> Yc[NY_], Vc[NY_], Yn[NY_], Vn[NY_], YN[NY_], u[NY_];
  cx<T> k[8][NY_];
  cx<T> spm[NP_];
  Rng rng;
  int64_t id;
  int task;
  T s, err, scale, residual;
  int tstepQ, streak, step, ministep, stage, attempt, it, phase, code;
  int n_ivp, n_newton;
};

template <typename T, int NY_>
__device__ __forceinline__ void draw_patch(Rng& r, double range, cx<T>* u) {
#pragma unroll 1
  for (int i = 0; i < NY_; ++i) {
    double re = 2.0 * range * r.uniform() - range;
    double im = 2.0 * range * r.uniform() - range;
    u[i] = cx<T>(T(re), T(im));
  }
}

template <typename T>
__device__ __forceinline__ T vnorm(const cx<T>* v, int n) {
  T s = T(0);
#pragma unroll 1
  for (int i = 0; i < n; ++i) s += cnorm2(v[i]);
  return sqrt(s);
}

// sum_{l < n} w[l] * s * k[l][e], accumulated from the last term to the first as the
// reference's nested .add() chains do (rungekutta.cu:40-122).
template <typename T, int NY_>
__device__ __forceinline__ cx<T> comb(const double* w, T s, const cx<T> (*k)[NY_], int n, int e) {
  cx<T> acc(T(0));
  bool first = true;
  for (int l = n - 1; l >= 0; --l) {
    if (w[l] == 0.0) continue;
    cx<T> term = (T(w[l]) * s) * k[l][e];
    acc = first ? term : term + acc;
    first = false;
  }
  return acc;
}

// Hand the path to the corrector (htpytrack.cu:135-154) or to sharpening
// (:194-213): YN starts from the prediction Yn.
template <typename T, int NY_, int NP_>
__device__ __forceinline__ void begin_newton(PathState<T, NY_, NP_>& P, int phase) {
#pragma unroll 1
  for (int e = 0; e < NY_; ++e) P.YN[e] = P.Yn[e];
  P.residual = T(100);
  P.it = 0;
  P.phase = phase;
}

template <class S>
__device__ void finish_path(const TrackArgs& a, int64_t id, int task, int code, cd* Yf, const cd* fpm);

// The task arrays in the working precision (FP32 copies are prepared by the host; the
// FP32 stage exists for Stephenson II only).
template <typename T, int NP_> struct TaskFpm;
template <int NP_> struct TaskFpm<double, NP_> {
  __device__ static const cx<double>* get(const TrackArgs& a, int task) { return a.fpm + (size_t)task * NP_; }
};
template <int NP_> struct TaskFpm<float, NP_> {
  __device__ static const cx<float>* get(const TrackArgs& a, int task) { return a.fpm_lo + (size_t)task * NP_; }
};
template <typename T> __device__ __forceinline__ cx<T> task_gamma(const TrackArgs& a, int task);
template <> __device__ __forceinline__ cx<double> task_gamma<double>(const TrackArgs& a, int task) {
  return a.gamma[task];
}
template <> __device__ __forceinline__ cx<float> task_gamma<float>(const TrackArgs& a, int task) {
  return a.gamma_lo[task];
}

template <typename T, int NY_, int NP_>
__device__ void save_handoff(const TrackArgs& a, const PathState<T, NY_, NP_>& P, int reason) {
  static_assert(NY_ <= NY, "hand-off records hold at most Stephenson II's 23-entry path states");
  Handoff& h = a.handoff[P.id];
#pragma unroll 1
  for (int e = 0; e < NY_; ++e) {
    h.Yc[e] = cd(P.Yc[e]);
    h.Vc[e] = cd(P.Vc[e]);
    h.u[e] = cd(P.u[e]);
  }
  h.s = double(P.s);
  h.rng_index = P.rng.index;
  h.streak = P.streak; h.step = P.step; h.ministep = P.ministep; h.tstepQ = P.tstepQ;
  h.n_ivp = P.n_ivp; h.n_newton = P.n_newton; h.reason = reason; h.code = 0;
  if (a.counters) { atomicAdd(&a.counters[12], 1ull); atomicAdd(&a.counters[15 + reason], 1ull); }
  const unsigned long long slot = atomicAdd(a.handoff_count, 1ull);
  a.handoff_list[slot] = P.id;
}

// S: the system (SysStephenson2 or a generated plug-in): NV_ unknowns, NZ_ = NV_ + 1
// homogeneous unknowns, NY_ = NV_ + 2 path-state entries, NP_ parameters; the linear
// systems are NY_ x NY_ with leading dimension LD_.
template <int MODE, typename T, class S>
__global__ void __launch_bounds__(FRG_TRACK_THREADS)
track_kernel(TrackArgs a) {
  constexpr int NV_ = S::NV, NZ_ = NV_ + 1, NY_ = NV_ + 2, NP_ = S::NP, LD_ = NY_ + 1;
  const frg_config& c = a.cfg;
  constexpr bool LO = (MODE == MODE_LO);
  const T newt_tol = LO ? T(c.newt_tol_lo) : T(c.newt_tol);
  PathState<T, NY_, NP_> P;
  cx<T> Ye[NY_], q[NP_], dq[NP_], F[NZ_], b[NY_], x[NY_];
  cx<T> M[NY_ * LD_];
  P.phase = PH_FETCH;
  unsigned long long fp64_solves = 0;
  const int64_t nqueue = (MODE == MODE_RESUME) ? (int64_t)*a.handoff_count : a.npaths;

  for (;;) {
    // ------------------------------------------------------------------ fetch
    if (P.phase == PH_FETCH) {
      const int64_t qi = (int64_t)atomicAdd(a.queue, 1ull);
      if (qi >= nqueue) break;
      const int64_t id = (MODE == MODE_RESUME) ? a.handoff_list[qi] : qi;
      P.id = id;
      int lo = 0, hi = a.ntasks - 1;  // task of this path
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (a.task_start[mid] <= id) lo = mid; else hi = mid - 1;
      }
      P.task = lo;
      // Start system (frg.cu:54): the stream of path id; TrackPath receives the same
      // fresh state (frg.cu:57, by value), so its draws restart at index 0.
      P.rng.seed = a.seed; P.rng.stream = (uint64_t)(id + c.path_offset); P.rng.index = 0;
      cd spt[NV_], spm[NP_];
      S::start(P.rng, c.start_dist, c.start_range, spt, spm);
#pragma unroll 1
      for (int e = 0; e < NP_; ++e) P.spm[e] = cx<T>(spm[e]);
      P.code = 0; P.stage = 0; P.attempt = 0; P.it = 0; P.residual = T(100); P.err = T(0); P.scale = T(0);
      if (MODE == MODE_RESUME) {
        const Handoff& h = a.handoff[id];
#pragma unroll 1
        for (int e = 0; e < NY_; ++e) { P.Yc[e] = cx<T>(h.Yc[e]); P.Vc[e] = cx<T>(h.Vc[e]); P.u[e] = cx<T>(h.u[e]); }
        P.s = T(h.s); P.rng.index = h.rng_index;
        P.streak = h.streak; P.step = h.step; P.ministep = h.ministep; P.tstepQ = h.tstepQ;
        P.n_ivp = h.n_ivp; P.n_newton = h.n_newton;
        P.phase = PH_RK;
      } else {
        P.rng.index = 0;
#pragma unroll 1
        for (int e = 0; e < NV_; ++e) P.Yc[e] = cx<T>(spt[e]);
        P.Yc[NV_] = cx<T>(T(1));
        P.Yc[NV_ + 1] = cx<T>(T(0));
        draw_patch<T, NY_>(P.rng, c.patch_range, P.u);
        switch_patch<T, NY_>(P.u, P.Yc, P.Yc);
        draw_patch<T, NY_>(P.rng, c.patch_range, P.Vc);
        P.s = T(c.s_init); P.tstepQ = 0; P.streak = c.caution_steps - 1; P.step = 0; P.ministep = 0;
        P.n_ivp = 0; P.n_newton = 0;
        P.phase = PH_TANGENT0;
      }
    }

    // -------------------------------------------------- set up the linear step
    const cx<T>* fpmT = TaskFpm<T, NP_>::get(a, P.task);
    const cx<T> gamma = task_gamma<T>(a, P.task);
    const bool newton = (P.phase == PH_NEWTON || P.phase == PH_SHARP);
    bool tstep = false;
    const cx<T>* patch = P.Vc;
    if (P.phase == PH_TANGENT0) {
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) Ye[e] = P.Yc[e];
    } else if (P.phase == PH_RK) {
      tstep = P.tstepQ != 0;
      const int st = P.stage;
      if (st == 0) {
#pragma unroll 1
        for (int e = 0; e < NY_; ++e) Ye[e] = P.Yc[e];
      } else {
        patch = P.k[st - 1];
#pragma unroll 1
        for (int e = 0; e < NY_; ++e) Ye[e] = P.Yc[e] + comb<T, NY_>(c_dpA[st], P.s, P.k, st, e);
      }
    } else {
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) Ye[e] = P.YN[e];
    }

    // ------------------------------------------------------ the linear step
    params_at<T, NP_>(Ye[NY_ - 1].re, P.spm, fpmT, gamma, q, dq);
    if (MODE != MODE_LO) fp64_solves++;
    S::template rows<T, LD_>(Ye, q, dq, M, newton ? F : nullptr);
    // row NV_: the projective patch u (htpysupport.cu:139-142); row NV_ + 1: the velocity patch
#pragma unroll 1
    for (int e = 0; e < NY_; ++e) { M[NV_ * LD_ + e] = P.u[e]; M[(NV_ + 1) * LD_ + e] = patch[e]; }
    T hnorm = T(0), ratio;
    if (newton) {
      cx<T> d(T(0));
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) d = cfma(P.u[e], Ye[e], d);
      F[NV_] = d - cx<T>(T(1));
      hnorm = vnorm(F, NZ_);
      row_scale<T, NY_, LD_>(M, NZ_, F);
#pragma unroll 1
      for (int e = 0; e < NZ_; ++e) b[e] = -F[e];
      b[NZ_] = cx<T>(T(0));
      const T tgoal = (P.phase == PH_SHARP) ? T(1) : P.Yn[NY_ - 1].re;
      ratio = lu_solve<T, NY_, LD_>(M, b, x, NZ_, true, cx<T>(tgoal - Ye[NY_ - 1].re));
      P.n_newton++;
    } else {
      row_scale<T, NY_, LD_>(M, NZ_, nullptr);
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) b[e] = cx<T>(T(0));
      b[NY_ - 1] = cx<T>(T(1));
      ratio = lu_solve<T, NY_, LD_>(M, b, x, NY_, false, cx<T>(T(0)));
      // normalise the tangent (htpysupport.cu:285-296): unit length with real
      // dt/ds, or dt = 1 when stepping in t. conj(x22)/|x22| is the reference's
      // (cos theta, -sin theta) with theta = arg(x22).
      cx<T> sc;
      if (!tstep) {
        const T ax = sqrt(cnorm2(x[NY_ - 1]));
        sc = cx<T>(x[NY_ - 1].re, -x[NY_ - 1].im) * (T(1) / (ax * vnorm(x, NY_)));
      } else {
        sc = cinv(x[NY_ - 1]);
      }
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) x[e] = sc * x[e];
      x[NY_ - 1].im = T(0);
      P.n_ivp++;
    }

    // ------------------------------------------------------------- transitions
    bool finished = false;
    int handoff = 0;
    const cx<T>* final_src = P.Yc;  // the reference's Yc aliases Yfinal (htpytrack.cu:46)
    if (LO && !(ratio <= T(c.cond_switch))) {
      handoff = 2;  // ill-conditioned (or non-finite) step: continue in FP64 from Yc
    } else if (P.phase == PH_TANGENT0) {
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) P.Vc[e] = x[e];
      if (c.max_steps == 0) { P.code = 1; finished = true; }
      P.stage = 0;
      P.phase = PH_RK;
    } else if (P.phase == PH_RK) {
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) P.k[P.stage][e] = x[e];
      if (++P.stage == 8) {
        P.stage = 0;
        // error estimate and step factor (rungekutta.cu:99-112), prediction (:115-122)
        T es = T(0);
#pragma unroll 1
        for (int e = 0; e < NY_; ++e) {
          es += cnorm2(comb<T, NY_>(c_dpE, P.s, P.k, 8, e));
          P.Yn[e] = P.Yc[e] + comb<T, NY_>(c_dpB, P.s, P.k, 8, e);
          P.Vn[e] = P.k[7][e];
        }
        P.err = sqrt(es);
        P.scale = (P.err > T(10e-17)) ? T(0.8) * pow(T(c.rk_tol) / P.err, T(1) / T(6)) : T(5);
        if (P.scale > T(5)) P.scale = T(5);
        if (P.ministep++ == c.max_ministeps) { P.code = 2; finished = true; }
        else if (P.err <= T(c.rk_tol)) {
          const T tn = P.Yn[NY_ - 1].re;
          if (LO && tn > T(1.0 - c.nudge_trigger)) handoff = 5;  // the endgame runs in FP64
          else if (tn <= T(1.0 - c.nudge_trigger)) { P.attempt = 0; begin_newton(P, PH_NEWTON); }
          else if (fabs(T(1) - tn) < T(c.sharp_trigger)) { P.attempt = 0; begin_newton(P, PH_SHARP); }
          else { P.tstepQ = 1; P.s = T(1) - P.Yc[NY_ - 1].re; }  // land on t = 1 (htpytrack.cu:120-123)
        } else {
          if (P.s <= T(c.s_min)) {
            if (LO) handoff = 4; else { P.code = 3; finished = true; }
          } else {
            P.s *= P.scale;
            if (P.s < T(c.s_min)) P.s = T(c.s_min * 0.9);
            P.streak = 0;
          }
        }
      }
    } else {
      // one corrector or sharpening iteration (htpysupport.cu:427-492)
      const bool sharp = (P.phase == PH_SHARP);
      const int max_its = sharp ? c.sharp_its : c.newt_its;
      const T tol = sharp ? T(c.sharp_tol) : newt_tol;
      const int restype = sharp ? c.sharp_residual : c.newt_residual;
      bool done = false;
      if (restype == 0 && P.it > 0) {
        // |H| at the current point is the residual of the previous update
        P.residual = hnorm;
        if (!(P.it < max_its && P.residual > tol)) done = true;
      }
      if (!done) {
#pragma unroll 1
        for (int e = 0; e < NY_; ++e) P.YN[e] += x[e];
        P.it++;
        if (restype != 0) {
          P.residual = vnorm(x, NY_);
          if (!(P.it < max_its && P.residual > tol)) done = true;
        }
      }
      if (done) {
        if (!sharp) {
          if (P.ministep++ == c.max_ministeps) { P.code = 2; finished = true; }
          else if (P.residual < newt_tol) {
            if (fabs(T(1) - P.Yn[NY_ - 1].re) < T(c.sharp_trigger)) { P.attempt = 0; begin_newton(P, PH_SHARP); }
            else {
              // accept the step (htpytrack.cu:176-183)
#pragma unroll 1
              for (int e = 0; e < NY_; ++e) { P.Yc[e] = P.YN[e]; P.Vc[e] = P.Vn[e]; }
              P.streak++;
              if (P.streak < c.caution_steps && P.scale > T(1)) P.scale = T(1);
              P.s *= P.scale;
              if (P.s > T(c.s_max)) P.s = T(c.s_max);
              else if (P.s < T(c.s_min)) P.s = T(c.s_min * 0.9);
              P.step++;
              if (P.step == c.max_steps) { P.code = 1; finished = true; }
              else if (LO && P.Yc[NY_ - 1].re >= T(c.t_switch)) handoff = 1;
              else { P.stage = 0; P.phase = PH_RK; }
            }
          } else {
            // new random patch and retry (htpytrack.cu:145-153)
            draw_patch<T, NY_>(P.rng, c.patch_range, P.u);
            switch_patch<T, NY_>(P.u, P.Yn, P.Yn);
            if (++P.attempt < c.newt_attempts) begin_newton(P, PH_NEWTON);
            else if (P.s <= T(c.s_min)) {
              if (LO) handoff = 3; else { P.code = 4; finished = true; }
            } else {
              P.s *= T(0.5);
              if (P.s < T(c.s_min)) P.s = T(c.s_min * 0.9);
              P.streak = 0;
              P.stage = 0;
              P.phase = PH_RK;
            }
          }
        } else {
          final_src = P.YN;
          if (P.ministep++ == c.max_ministeps) { P.code = 2; finished = true; }
          else if (P.residual < T(c.sharp_tol)) { P.code = 0; finished = true; }
          else {
            draw_patch<T, NY_>(P.rng, c.patch_range, P.u);
            switch_patch<T, NY_>(P.u, P.Yn, P.Yn);
            if (++P.attempt < c.sharp_attempts) begin_newton(P, PH_SHARP);
            else { P.code = 5; finished = true; }
          }
        }
      }
    }

    if constexpr (LO) {
      if (handoff) {
        save_handoff(a, P, handoff);
        P.phase = PH_FETCH;
        continue;
      }
    }

    // ---------------------------------------------------------------- finish
    if (finished) {
      cd Yf[NY_];
#pragma unroll 1
      for (int e = 0; e < NY_; ++e) Yf[e] = cd(final_src[e]);
      finish_path<S>(a, P.id, P.task, P.code, Yf, a.fpm + (size_t)P.task * NP_);
      if (a.work) {
        a.work[(size_t)P.id * 3 + 0] = P.n_ivp;
        a.work[(size_t)P.id * 3 + 1] = P.n_newton;
        a.work[(size_t)P.id * 3 + 2] = P.step;
      }
      if (a.counters) {
        atomicAdd(&a.counters[8], (unsigned long long)P.n_ivp);
        atomicAdd(&a.counters[9], (unsigned long long)P.n_newton);
        atomicAdd(&a.counters[10], (unsigned long long)P.step);
      }
      P.phase = PH_FETCH;
    }
  }
  // FP64 linear steps of this thread (all of them for MODE_PLAIN and MODE_RESUME)
  if (a.counters && fp64_solves) atomicAdd(&a.counters[11], fp64_solves);
}

// Write a finished path: the tracked endpoint (optional), the finite check, the
// dehomogenized canonical root (frg.cu:44-46, :59-68), its code, and the
// row-scaled residual of the target system at the root.
template <class S>
__device__ void finish_path(const TrackArgs& a, int64_t id, int task, int code, cd* Yf, const cd* fpm) {
  constexpr int NV_ = S::NV, NZ_ = NV_ + 1, NY_ = NV_ + 2, NP_ = S::NP, LD_ = NY_ + 1;
  const frg_config& c = a.cfg;
  if (a.yfinal) {
#pragma unroll 1
    for (int e = 0; e < NY_; ++e) a.yfinal[(size_t)id * NY_ + e] = Yf[e];
  }
  if (code == 0 && c.inf_tol > 0.0) {
    double zmax = 0.0;
#pragma unroll 1
    for (int e = 0; e < NV_; ++e) zmax = fmax(zmax, sqrt(cnorm2(Yf[e])));
    if (sqrt(cnorm2(Yf[NV_])) < c.inf_tol * zmax) code = FRG_CODE_INFINITE;
  }
  cd ud[NY_];
#pragma unroll 1
  for (int e = 0; e < NY_; ++e) ud[e] = cd(0.0);
  ud[NV_] = cd(1.0);
  switch_patch<double, NY_>(ud, Yf, Yf);
  cd root[NV_];
  S::canonical(Yf, fpm, root);
#pragma unroll 1
  for (int e = 0; e < NV_; ++e) a.roots[(size_t)id * NV_ + e] = root[e];
  a.codes[id] = code;
  if (a.counters) atomicAdd(&a.counters[code & 7], 1ull);
  if (a.resid) {
    cd Y[NY_], q[NP_], dq[NP_], F[NZ_];
    cd M[NY_ * LD_];
#pragma unroll 1
    for (int e = 0; e < NV_; ++e) Y[e] = root[e];
    Y[NV_] = cd(1.0);
    Y[NV_ + 1] = cd(1.0);
#pragma unroll 1
    for (int e = 0; e < NP_; ++e) { q[e] = fpm[e]; dq[e] = cd(0.0); }
    S::template rows<double, LD_>(Y, q, dq, M, F);
    double r = 0.0;
#pragma unroll 1
    for (int i = 0; i < NV_; ++i) {
      double mx = 0.0;
#pragma unroll 1
      for (int e = 0; e < NZ_; ++e) mx = fmax(mx, fmax(fabs(M[i * LD_ + e].re), fabs(M[i * LD_ + e].im)));
      const double ri = sqrt(cnorm2(F[i])) / mx;
      r = (ri == ri) ? fmax(r, ri) : INFINITY;  // a non-finite row makes the residual infinite
    }
    a.resid[id] = r;
  }
}

}  // namespace frg

namespace {
__global__ void to_float_kernel(const cx<double>* in, cx<float>* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cx<float>(in[i]);
}
__global__ void to_df_kernel(const cx<double>* in, cx<df>* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cx<df>(df(in[i].re), df(in[i].im));
}

template <int MODE, typename T, class S = frg::SysStephenson2>
cudaError_t launch(const frg::TrackArgs& args, int grid, cudaStream_t stream) {
  frg::track_kernel<MODE, T, S><<<grid, FRG_TRACK_THREADS, 0, stream>>>(args);
  return cudaGetLastError();
}
}  // namespace

cudaError_t frg_launch_track(int mode, const frg::TrackArgs& args, int grid, cudaStream_t stream) {
  if (args.cfg.system != 0) {  // plug-in systems: plain FP64, or the FP32 stage and the FP64 resume
    switch (args.cfg.system) {
#define FRG_PLUGIN_LAUNCH(id, name, S)                                                 \
  case id:                                                                            \
    switch (mode) {                                                                   \
      case frg::MODE_PLAIN: return launch<frg::MODE_PLAIN, double, S>(args, grid, stream); \
      case frg::MODE_LO: return launch<frg::MODE_LO, float, S>(args, grid, stream);         \
      case frg::MODE_RESUME: return launch<frg::MODE_RESUME, double, S>(args, grid, stream); \
      default: return cudaErrorInvalidValue;                                          \
    }
      FRG_PLUGIN_LIST(FRG_PLUGIN_LAUNCH)
#undef FRG_PLUGIN_LAUNCH
      default: return cudaErrorInvalidValue;
    }
  }
  switch (mode) {
    case frg::MODE_PLAIN: return launch<frg::MODE_PLAIN, double>(args, grid, stream);
    case frg::MODE_LO: return launch<frg::MODE_LO, float>(args, grid, stream);
    case frg::MODE_RESUME: return launch<frg::MODE_RESUME, double>(args, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t frg_launch_to_float(const cx<double>* in, cx<float>* out, int n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  to_float_kernel<<<(n + 127) / 128, 128, 0, stream>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t frg_launch_to_df(const cx<double>* in, cx<df>* out, int n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  to_df_kernel<<<(n + 127) / 128, 128, 0, stream>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t frg_track_occupancy(int mode, int* blocks_per_sm) {
  switch (mode) {
    case frg::MODE_PLAIN:
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          blocks_per_sm, frg::track_kernel<frg::MODE_PLAIN, double, frg::SysStephenson2>, FRG_TRACK_THREADS, 0);
    case frg::MODE_LO:
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          blocks_per_sm, frg::track_kernel<frg::MODE_LO, float, frg::SysStephenson2>, FRG_TRACK_THREADS, 0);
    case frg::MODE_RESUME:
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          blocks_per_sm, frg::track_kernel<frg::MODE_RESUME, double, frg::SysStephenson2>, FRG_TRACK_THREADS, 0);
    default: return cudaErrorInvalidValue;
  }
}

template <int MODE, typename T, class S>
static cudaError_t occ(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, frg::track_kernel<MODE, T, S>,
                                                       FRG_TRACK_THREADS, 0);
}

cudaError_t frg_track_occupancy_system(int system, int mode, int* blocks_per_sm) {
  if (system == 0) return frg_track_occupancy(mode, blocks_per_sm);
  switch (system) {
#define FRG_PLUGIN_OCC(id, name, S)                                             \
  case id:                                                                     \
    switch (mode) {                                                            \
      case frg::MODE_PLAIN: return occ<frg::MODE_PLAIN, double, S>(blocks_per_sm); \
      case frg::MODE_LO: return occ<frg::MODE_LO, float, S>(blocks_per_sm);         \
      case frg::MODE_RESUME: return occ<frg::MODE_RESUME, double, S>(blocks_per_sm); \
      default: return cudaErrorInvalidValue;                                   \
    }
    FRG_PLUGIN_LIST(FRG_PLUGIN_OCC)
#undef FRG_PLUGIN_OCC
    default: return cudaErrorInvalidValue;
  }
}

int frg_system_dims(int system, const char** name, int* nv, int* np) {
  switch (system) {
    case 0: *name = "stephenson2"; *nv = frg::NV; *np = frg::NP; return 1;
#define FRG_PLUGIN_DIMS(id, nm, S) \
  case id: *name = nm; *nv = S::NV; *np = S::NP; return 1;
    FRG_PLUGIN_LIST(FRG_PLUGIN_DIMS)
#undef FRG_PLUGIN_DIMS
    default: return 0;
  }
}

int frg_system_count() { return 1 + FRG_NUM_PLUGINS; }
