// Internal interface between the C ABI (frg_capi.cu) and the tracking kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/frg_gb300.h"
#include "frg_complex.cuh"
#include "frg_df.cuh"
#include "frg_mlp.cuh"

#ifndef FRG_TRACK_THREADS
#define FRG_TRACK_THREADS 64
#endif
#ifndef FRG_TEAM_THREADS
#define FRG_TEAM_THREADS 64
#endif

namespace frg {

// Saved state of a path handed from the FP32 stage to the FP64 stage: what the
// reference's tracker carries across loop iterations (htpytrack.cu:36-77).
struct Handoff {
  cx<double> Yc[23], Vc[23], u[23];
  double s;
  uint64_t rng_index;
  int streak, step, ministep, tstepQ, n_ivp, n_newton, reason, code;  // reason 6: finished with code
  int bounces, pad;  // times the path returned from FP64 to FP32
};

// Device-side arguments of one tracking launch. All arrays are device memory.
constexpr int FRG_START_STRIDE = 51;
// counters: codes[8], ivp, newton, steps, fp64 solves, handoffs, hand-backs, -, -, handoff
// reasons 1..6 at [16..21], refinement solves and warp steps at [22..23], kernel cycles at
// [24..35], retired paths at [36], FP32-stage refinement-residual cycles at [37],
// FP64-segment histogram at [40..45], longest FP64 segment at [46]
#define FRG_NCOUNTERS 48

struct TrackArgs {
  frg_config cfg;
  const cx<double>* fpm;        // ntasks x 30 target parameters
  const cx<double>* gamma;      // ntasks
  const cx<float>* fpm_lo;      // FP32 copies for the FP32 stage
  const cx<float>* gamma_lo;
  const cx<df>* fpm_df;         // double-float copies for the FP32 stage's refinement residuals
  const cx<df>* gamma_df;
  const int64_t* task_start;    // ntasks + 1 prefix sums of paths per task
  int ntasks;
  int64_t npaths;               // paths of one round
  uint64_t seed;
  // Paths are addressed by a global index gid = round * npaths + (index within the round):
  // records, lists and outputs use gid; the random stream, start values and task use the
  // index within the round; task parameters and gammas are indexed by round * ntasks + task.
  // A single call is round 0 (gid = index within the round).
  int64_t round_base;           // gid of this launch's first fresh path (round * npaths)
  const uint64_t* seeds;        // per-round seeds (null: every path uses `seed`)
  int carry;                    // FP32 stage: lo_list holds paths carried over from an earlier
                                // round's FP64 launch, taken before this round's fresh paths
  unsigned long long* queue;    // work-queue head, zeroed before launch
  cx<double>* roots;            // npaths x 21
  int32_t* codes;               // npaths
  cx<double>* yfinal;           // npaths x 23, optional
  double* resid;                // npaths, optional
  int32_t* work;                // npaths x 3 (ivp solves, newton iterations, steps), optional
  unsigned long long* counters; // FRG_NCOUNTERS counters (layout above)
  const cx<double>* starts;     // npaths x FRG_START_STRIDE start values (null: generated inline)
  Handoff* handoff;             // npaths slots (mixed precision)
  int64_t* handoff_list;        // ids of paths handed to the FP64 kernel
  unsigned long long* handoff_count;
  const int64_t* lo_list;       // FP32 kernel: paths to resume from their saved state (null: fresh paths)
  const unsigned long long* lo_count;
  int64_t* back_list;           // FP64 kernel: paths handed back to FP32 (null: none, e.g. the last round)
  unsigned long long* back_count;
  int lo_keep_ill;              // FP32 kernel: 1 = no hand-off for ill-conditioned steps (last round)
  float* feat;                  // optional: FRG_MLP_IN features per checkpoint, feat_max checkpoints per path
  int32_t* nfeat;               // checkpoints written per path (zeroed before launch)
  int feat_max;
  int feat_every;               // checkpoint every this many accepted steps (features and retirement)
  MlpDevice mlp;                // early-retirement network (mlp.w null: off)
};

}  // namespace frg

// mode: 0 plain FP64, 1 FP32 stage with handoff, 2 FP64 resume of handed-off paths
cudaError_t frg_launch_track(int mode, const frg::TrackArgs& args, int grid, cudaStream_t stream);
cudaError_t frg_track_occupancy(int mode, int* blocks_per_sm);
cudaError_t frg_launch_team(int mode, const frg::TrackArgs& args, int grid, cudaStream_t stream);
// GenerateStart for every path into args.starts (FRG_START_STRIDE complex per path:
// the 21 start unknowns, then the 30 start parameters)
cudaError_t frg_launch_starts(const frg::TrackArgs& args, cx<double>* starts, cudaStream_t stream);
cudaError_t frg_team_occupancy(int mode, int* blocks_per_sm);
cudaError_t frg_launch_to_float(const cx<double>* in, cx<float>* out, int n, cudaStream_t stream);
cudaError_t frg_launch_to_df(const cx<double>* in, cx<df>* out, int n, cudaStream_t stream);
// Occupancy of the thread kernel of `system` (0 = Stephenson II, k = plug-in k) in `mode`
// (0 plain FP64, 1 FP32 stage, 2 FP64 resume).
cudaError_t frg_track_occupancy_system(int system, int mode, int* blocks_per_sm);
// Name, unknowns and parameters of `system`; 0 for an unknown id. Host only.
int frg_system_dims(int system, const char** name, int* nv, int* np);
// Number of systems: Stephenson II and the generated plug-ins.
int frg_system_count();
// Validates a run configuration (every field frg_create and frg_set_config accept);
// ctx may be null, otherwise it receives the error text.
frg_status frg_check_config(frg_ctx* ctx, const frg_config* c);
