/*
 * frg_gb300: GB300-native finite-root-generation path tracker, C ABI.
 *
 * The reference (mplecnik/Finite_Root_Generation) has no plugin or FFI layer; its
 * seam is the set of calls its driver makes each round (frg.cu:351-514):
 *   InitRandStates + Homotopy kernels          (frg.cu:30-124, launched :361, :374)
 *   cudaMemcpy of roots and error codes        (frg.cu:389, :398)
 *   thrust::sort_by_key on Re(root[0])          (frg.cu:432-435)
 *   SortingDeletingMerging                     (frgsupport.cuh:7, called frg.cu:440)
 *   LambertW coverage estimate                 (frgsupport.cuh:9, called frg.cu:463-464)
 *   fptColl / errorCodesAgr persistence        (frg.cu:295-336, :472-480)
 * Each entry point below names the reference interface it replaces.
 *
 * Conventions kept from the reference:
 *   - complex numbers are interleaved (re, im) doubles (cuDoubleComplex, classes.cuh:24-25);
 *   - a root is 21 complex values [A,B,C,D,F,G,H, Ac..Hc, U1..U7] = 336 bytes
 *     (Vect<nV>, htpykinematics.cuh:8), dehomogenized and in canonical cognate form;
 *   - a task (target parameter set) is 30 complex values
 *     [P0..P7, Pc0..Pc7, Q1..Q7, Qc1..Qc7] (Vect<nP>, frg.cu:147-178);
 *   - per-path codes: 0 success, 1 max steps, 2 max ministeps, 3 predictor step
 *     below s_min, 4 corrector failed at s_min, 5 sharpening failed
 *     (htpytrack.cu:85,95,100,159,216), 6 duplicate (frgsupport.cu:8), plus
 *     7 = tracked to an infinite root (only when frg_config.inf_tol > 0); code 2 also
 *     marks paths ended by fp64_budget or by the early-retirement network;
 *   - buffers are owned by the caller and may be host or device memory.
 *
 * Errors: functions return frg_status; FRG_OK == 0, negative values are argument,
 * allocation or CUDA errors whose text frg_last_error() returns. One context per
 * host thread; contexts share no state.
 */
#ifndef FRG_GB300_H
#define FRG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FRG_NV 21 /* unknowns per root (htpykinematics.cuh:8) */
#define FRG_NP 30 /* parameters per task (htpykinematics.cuh:9) */
#define FRG_NY 23 /* tracked state: 21 unknowns, homogenizer, t */

typedef enum {
  FRG_OK = 0,
  FRG_ERR_ARG = -1,
  FRG_ERR_ALLOC = -2,
  FRG_ERR_CUDA = -3,
  FRG_ERR_IO = -4,
  FRG_ERR_TIMEOUT = 1
} frg_status;

enum { FRG_CODE_OK = 0, FRG_CODE_MAX_STEPS = 1, FRG_CODE_MAX_MINISTEPS = 2, FRG_CODE_RK_SMIN = 3,
       FRG_CODE_NEWTON_SMIN = 4, FRG_CODE_SHARPEN = 5, FRG_CODE_DUPLICATE = 6, FRG_CODE_INFINITE = 7 };

enum { FRG_PREC_FP64 = 0, FRG_PREC_MIXED = 1 };
enum { FRG_START_UNIFORM = 0, FRG_START_NORMAL = 1 };
enum { FRG_GAMMA_FIXED = 0, FRG_GAMMA_RANDOM = 1 };
enum { FRG_KERNEL_TEAM = 0, FRG_KERNEL_THREAD = 1 };

/* Run configuration. frg_config_default() fills the reference's compile-time
 * constants: tracker settings htpytrack.cu:9-31, start range frgkinematics.cu:7-8,
 * gamma frg.cu:41, duplicate tolerance frgsupport.cu:7. */
typedef struct frg_config {
  double s_init, s_max, s_min, rk_tol;
  int caution_steps;
  int newt_its;
  double newt_tol;
  int newt_residual; /* 0: |H|, 1: |dY| */
  int newt_attempts;
  int sharp_its;
  double sharp_tol;
  int sharp_residual;
  int sharp_attempts;
  double sharp_trigger, nudge_trigger;
  int max_steps, max_ministeps;
  double patch_range;   /* patches uniform in (-r, r)^2 */
  int start_dist;       /* FRG_START_UNIFORM (reference) or FRG_START_NORMAL */
  double start_range;   /* uniform start range r: values in (-r, r)^2 */
  int gamma_mode;       /* FRG_GAMMA_FIXED uses gamma_re/im; FRG_GAMMA_RANDOM draws e^{i phi} per task */
  double gamma_re, gamma_im;
  double dup_tol;       /* absolute per-component duplicate tolerance */
  int precision;        /* FRG_PREC_FP64 (reference arithmetic) or FRG_PREC_MIXED */
  double t_switch;      /* mixed, lo_endgame = 0: FP64 tracking once t exceeds this */
  double cond_switch;   /* mixed: a step whose condition estimate (the elimination's pivot ratios)
                           exceeds this continues its path in FP64 */
  double inf_tol;       /* > 0: |Z0| / |Z| below this at t = 1 marks code 7 */
  int threads_per_block; /* 0 = tuned default */
  int blocks_per_sm;     /* 0 = tuned default */
  double newt_tol_lo;    /* mixed: corrector tolerance of the FP32 stage */
  int kernel_variant;    /* FRG_KERNEL_TEAM (8 lanes per path, default) or FRG_KERNEL_THREAD */
  int mixed_rounds;      /* mixed, team kernels: FP32/FP64 rounds; a path well conditioned again in
                            FP64 returns to FP32 in the next round (1 = no return) */
  int lo_refine;         /* mixed: 1 = the FP32 corrector refines on residuals in the point type
                            (lo_points) to newt_tol; 2 = the same, but a refined iteration whose
                            successor is predicted below newt_tol / 10 ends it; 3 = a corrector
                            whose FP32 update falls below newt_tol_lo is accepted without
                            refinement, one that stalls above it refines as in 1; 0 = it stops
                            at newt_tol_lo */
  int lo_endgame;        /* mixed: 1 = the FP32 stage (with refinement) also runs the endgame and
                            sharpening, FP64 only for ill-conditioned steps; 0 = FP64 from t_switch */
  int64_t path_offset;   /* random stream of local path i is path_offset + i: shards of one round
                            (path-index ranges on several GPUs) reproduce the single-GPU round */
  int fp64_budget;       /* mixed: a path that spends more FP64 solves than this in one FP64 launch
                            ends with code 2 (step limit); 0 = no limit */
  int lo_points;         /* mixed, team kernels: the FP32 stage keeps its points and refinement
                            residuals in 0 = FP64, 1 = double-float (FP32 pipes, larger code) */
  int fp64_segment;      /* mixed, mixed_rounds >= 2: FP64 solves after which a path returns to the
                            next round's FP32 kernel at its next accepted step (0 = 96) */
  int handback_good;     /* mixed, mixed_rounds >= 2: consecutive well-conditioned FP64 solves after
                            which a path returns to FP32 (0 = only after fp64_segment) */
  int lo_final;          /* mixed, mixed_rounds >= 2: 1 = the last round's FP32 kernel keeps paths
                            whose steps are ill conditioned (no hand-off for conditioning); paths
                            then use FP64 only for one bounded segment per earlier round */
  int carry_handback;    /* mixed, team kernels, frg_track_rounds: 1 = a path that is well
                            conditioned again in a round's FP64 launch (handback_good / fp64_segment)
                            continues in the FP32 launch of the round `depth` rounds later on the
                            same stream, so no launch is added; the last `depth` rounds finish
                            their paths in FP64. Per path the same computation as frg_track with
                            mixed_rounds = the rounds left on the path's stream; 0 = a handed-off
                            path stays in FP64 */
  int round_graph;       /* frg_track_rounds with carry_handback: 1 = every round's launches, on
                            every stream, are captured into one CUDA graph and launched once (the
                            same results); 0 = launched one by one */
  int system;            /* the polynomial system tracked: 0 = Stephenson II (the reference's
                            htpykinematics.cu, nV = 21, nP = 30); k >= 1 = generated plug-in k
                            (frg_system_info). A plug-in runs on the thread kernel
                            (kernel_variant THREAD), in FP64 or mixed precision (the FP32
                            stage handing paths to FP64), through frg_track,
                            frg_track_async and frg_track_rounds; its tasks are ntasks x np
                            parameters, its roots N x nv, its yfinal N x (nv + 2), and its roots
                            are reported as tracked (no cognate map) */
} frg_config;

/* A system the library tracks (frg_config.system). */
typedef struct frg_system_desc {
  char name[32];         /* "stephenson2" for system 0, the plug-in module's NAME otherwise */
  int nv;                /* unknowns of a root (affine) */
  int np;                /* parameters of a task */
} frg_system_desc;

/* Per-call counters (all paths of the call). */
typedef struct frg_stats {
  int64_t paths;
  int64_t codes[8];        /* number of paths ending with each code */
  int64_t ivp_solves;      /* 23x23 tangent solves (predictor stages + initial tangent) */
  int64_t newton_iters;    /* 22x22 corrector / sharpening solves */
  int64_t fp64_solves;     /* of the above, solves done in FP64 (mixed precision) */
  int64_t steps;           /* accepted steps */
  double track_ms;         /* device time of the tracking kernel(s) */
  double total_ms;         /* wall time of the call, copies included */
  int64_t handoffs;        /* mixed precision: paths continued in FP64 */
  double stage_ms[2];      /* device time of the FP32 stage and of the FP64 kernel */
  int64_t handoff_reason[6]; /* mixed: t_switch, ill-conditioned, corrector at s_min,
                                predictor at s_min, endgame entry, ended on a step limit */
  int64_t kernel_cycles[12]; /* team kernels, summed over warps: [0..5] FP32 stage, [6..11] FP64
                                kernel; per kernel the cycles in path fetch, step set-up, linear steps
                                and transitions, then warp steps and active-team steps */
  int64_t handbacks;       /* mixed: returns from FP64 to FP32 once well conditioned again */
  int64_t refine_solves;   /* mixed: FP32-stage corrector iterations on double-float residuals */
  int64_t refine_warp_steps; /* mixed: FP32-stage warp steps in which at least one path refined */
  double round_ms[32];     /* mixed: FP32-stage and FP64-stage times, interleaved, of mixed rounds
                              0..15 (frg_track) or of rounds 0..15 of the call (frg_track_rounds) */
  int64_t fp64_segment_hist[6]; /* mixed: paths leaving an FP64 launch after <100, <300, <1000, <3000,
                                   <10000, >=10000 FP64 solves in it */
  int64_t fp64_segment_max;     /* mixed: most FP64 solves one path spent in one FP64 launch */
  int64_t retired;              /* paths the early-retirement network ended (reported as code 2) */
  int64_t refine_cycles;        /* mixed: FP32-stage cycles (summed over warps) spent evaluating the
                                   double-float refinement residuals, part of kernel_cycles[2] */
} frg_stats;

typedef struct frg_ctx frg_ctx;

/* Fill cfg with the reference's defaults. */
frg_status frg_config_default(frg_config* cfg);

/* Describe system `system` (0 = Stephenson II, 1..frg_num_systems()-1 = the generated
 * plug-ins); FRG_ERR_ARG for an unknown id. The reference hard-wires one system
 * (nV = 21, nP = 30, htpykinematics.cuh:8-9); this replaces those constants. Host only,
 * no GPU needed. */
frg_status frg_system_info(int system, frg_system_desc* desc);
int frg_num_systems(void);

/* Create a context on CUDA device `device` (replaces the reference's implicit
 * device 0 and its cudaMalloc block, frg.cu:139, :201-236). */
frg_status frg_create(frg_ctx** ctx, const frg_config* cfg, int device);
void frg_destroy(frg_ctx* ctx);
const char* frg_last_error(const frg_ctx* ctx);
frg_status frg_set_config(frg_ctx* ctx, const frg_config* cfg);

/* Track paths (replaces InitRandStates + Homotopy + the two copies back,
 * frg.cu:30-124, :361-404). Path i of task k uses random stream
 * (sum of paths of earlier tasks) + i of `seed`; the reference's per-thread curand
 * subsequence i (frg.cu:32).
 *   fpm            ntasks x 30 complex target parameters (ntasks x np for a plug-in system)
 *   paths_per_task ntasks counts; total N = sum
 *   roots          out, N x 21 complex (canonical cognate, dehomogenized, frg.cu:59-68; a plug-in
 *                  system's N x nv roots are dehomogenized as tracked)
 *   codes          out, N int32
 *   yfinal         optional out, N x 23 complex tracked endpoints before dehomogenizing (N x (nv + 2))
 *   resid          optional out, N doubles: max |F_r| / max_c |dF_r/dZ_c| at the root
 *   stats          optional out
 * Pointers may be host or device memory (probed). Synchronous. */
frg_status frg_track(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                     uint64_t seed, double* roots, int32_t* codes, double* yfinal, double* resid,
                     frg_stats* stats);

/* Same, enqueued on `stream` (a cudaStream_t); device pointers only, returns
 * before the work completes. */
frg_status frg_track_async(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                           uint64_t seed, double* roots, int32_t* codes, double* yfinal, double* resid,
                           void* stream);

/* `nrounds` rounds of the reference driver's loop (frg.cu:351-514, one Homotopy launch
 * per round, seeds[r] in place of its time(NULL) reseed at :359) in one call, pipelined:
 * up to `depth` rounds are in flight on separate streams, so a round's long FP64 tail
 * overlaps the next rounds' tracking. per_round_tasks = 0: every round tracks the same
 * ntasks tasks (fpm: ntasks x 30 complex), as the reference's loop does; 1: round r
 * tracks its own task set (fpm: nrounds x ntasks x 30 complex, set r at r*ntasks*30),
 * e.g. a large batch of tasks split into rounds. Round r writes roots + r*N*21*2,
 * codes + r*N and resid + r*N (N = sum of paths_per_task); these are all device or all
 * host buffers (host copies are asynchronous when the host memory is pinned). stats
 * sums all rounds; track_ms spans the first launch to the last round's end. */
frg_status frg_track_rounds(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                            int nrounds, const uint64_t* seeds, int per_round_tasks, int depth, double* roots,
                            int32_t* codes, double* resid, frg_stats* stats);

/* Early retirement (no counterpart in the reference). A 32 -> 64 -> 64 -> 3 ReLU network
 * (BF16 weights, FP32 sums) scores a path's tracking features every `every` accepted
 * steps; a path whose probability of failing (no finite root with residual <= 1e-10)
 * reaches `threshold` is ended and reported as code 2. params: FP32 weights in the
 * layout of frg_mlp_param_count() (W1[64][32] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]);
 * mu, inv_sigma: the 32 features' standardisation. params = NULL switches it off. */
frg_status frg_set_mlp(frg_ctx* ctx, const float* params, const float* mu, const float* inv_sigma, float threshold,
                       int every);

/* frg_track (host or device outputs, no yfinal) that also records each path's
 * checkpoint features: up to max_checkpoints vectors of 32 floats per path, one every
 * `every` accepted steps, into features[N][max_checkpoints][32] (host), their count in
 * nfeat[N]. The training data of the early-retirement network. */
frg_status frg_track_features(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                              uint64_t seed, double* roots, int32_t* codes, double* resid, float* features,
                              int32_t* nfeat, int max_checkpoints, int every, frg_stats* stats);

/* The network's training and batch inference, with the library's own CUDA kernels on
 * the current device. X: n x 32 standardised features (host), y: classes 0 new root,
 * 1 fails, 2 duplicate root. frg_mlp_grad: mean class-weighted cross entropy and its
 * gradient with respect to the BF16-rounded weights (host outputs). frg_mlp_train:
 * Adam on shuffled mini-batches from `params` (all zero: He-normal start drawn from
 * `seed`); params is updated in place, epoch_loss (optional) gets each epoch's mean
 * loss. frg_mlp_predict: n x 3 class probabilities. */
int frg_mlp_param_count(void);
frg_status frg_mlp_grad(const float* X, const int32_t* y, int64_t n, const float* params, const float* class_w,
                        float* grad, double* loss);
frg_status frg_mlp_train(const float* X, const int32_t* y, int64_t n, const float* class_w, int epochs, int batch,
                         float lr, uint64_t seed, float* params, double* epoch_loss);
frg_status frg_mlp_predict(const float* X, int64_t n, const float* params, float* probs);

/* Plain FP64 tracking that allocates no device memory. No counterpart in the
 * reference: it is for callers that may not call cudaMalloc / cudaFree, such as code
 * hosted in a framework that owns all device memory through its own pool, or loops
 * that cannot afford cudaFree's device-wide synchronisation. The caller passes device
 * buffers for fpm, roots, codes and (optional) resid; cfg and paths_per_task are host
 * memory; cfg->precision must be FRG_PREC_FP64. The work runs on the current device,
 * enqueued on `stream` (a cudaStream_t, NULL for the legacy stream); the call returns
 * before it completes. The kernels' scratch (queue head, counters, per-task gamma and
 * path offsets) is a static device array of FRG_NOALLOC_SCRATCH_BYTES kept by every
 * GPU that loads the library until exit, so a call takes at most
 * FRG_NOALLOC_MAX_TASKS tasks (more returns FRG_ERR_ARG). The first call on a device
 * looks up the array's device address; make it before any stream capture. All calls
 * share the array: calls whose GPU work overlaps on one device race. cfg is checked
 * like frg_create's (a config frg_create refuses is refused here), and every buffer
 * must be device memory of the current device (or managed memory). Errors are
 * reported by the status alone (FRG_ERR_ARG for bad arguments, FRG_ERR_CUDA). */
#define FRG_NOALLOC_MAX_TASKS 1024
#define FRG_NOALLOC_SCRATCH_BYTES 32768
frg_status frg_track_noalloc(const frg_config* cfg, const double* fpm, int ntasks, const int64_t* paths_per_task,
                             uint64_t seed, double* roots, int32_t* codes, double* resid, void* stream);

/* ---- root collection (replaces SortingDeletingMerging, frgsupport.cu:10-215, and
 *      the thrust ordering of frg.cu:432-435). The host and device collections hold
 *      Stephenson II roots (21 complex, the fptColl layout); a plug-in system's roots
 *      are deduplicated by the caller. ---- */
typedef struct frg_coll frg_coll;

frg_status frg_coll_create(frg_coll** coll, double dup_tol);
void frg_coll_destroy(frg_coll* coll);
int64_t frg_coll_size(const frg_coll* coll);
/* Copy the sorted collection (size x 21 complex) to host memory `out`. */
frg_status frg_coll_get(const frg_coll* coll, double* out, int64_t capacity);
/* Merge one round of roots into the collection: successes (code 0) that duplicate a
 * collected root, or an earlier success of the round, within dup_tol in every real
 * component become code 6 in place; the others are added. Host memory. */
frg_status frg_coll_merge(frg_coll* coll, const double* roots, int32_t* codes, int64_t n);
/* Persistence in the reference's byte formats: fptColl = raw roots, 336 bytes each,
 * sorted; errorCodesAgr = int32 per trial, appended (frg.cu:295-336, :472-480). */
frg_status frg_coll_save(const frg_coll* coll, const char* fpt_coll_path);
frg_status frg_coll_load(frg_coll* coll, const char* fpt_coll_path);
frg_status frg_codes_append(const char* error_codes_path, const int32_t* codes, int64_t n);

/* ---- device-resident root collection: SortingDeletingMerging (frgsupport.cu:10-215)
 *      and the thrust ordering of frg.cu:432-435 on the GPU, across rounds, one
 *      collection per key (e.g. per task) ---- */
typedef struct frg_dcoll frg_dcoll;

/* A collection of at most `capacity` roots on `device` (device memory: 336 bytes per root
 * plus a hash table of 16 bytes per slot, 2 to 4 slots per root); dup_tol > 0. */
frg_status frg_dcoll_create(frg_dcoll** coll, int device, int64_t capacity, double dup_tol);
void frg_dcoll_destroy(frg_dcoll* coll);
/* Merge n roots (device memory: roots n x 21 complex, codes n int32, keys n int32 in
 * [0, 2^20) or NULL for key 0) on `stream`: the same marks as frg_coll_merge applied per
 * key -- a success (code 0) within dup_tol in every real component of a collected root
 * of its key, or of a lower-index success of the same call and key that is itself not a
 * duplicate, becomes code 6 in place; the others are collected. resid (n doubles, or
 * NULL): a success whose residual is above resid_max (or not a number) takes no part
 * (its code is left as it is). A root whose first component is not finite matches
 * nothing. Asynchronous; merges on one collection must be ordered (one stream, or
 * events). */
frg_status frg_dcoll_merge(frg_dcoll* coll, const double* roots, int32_t* codes, const double* resid,
                           double resid_max, const int32_t* keys, int64_t n, void* stream);
/* Roots collected so far (synchronizes `stream`); FRG_ERR_ALLOC if a merge ran out of
 * capacity (the roots past it were marked kept but not collected). */
frg_status frg_dcoll_size(frg_dcoll* coll, void* stream, int64_t* size);
/* Copy the collected roots (in collection order, not sorted) and their keys (optional)
 * to host memory; synchronizes the device. */
frg_status frg_dcoll_get(frg_dcoll* coll, double* roots, int32_t* keys, int64_t capacity);

/* ---- statistics (frgsupport.cu:220-272, frg.cu:463-464) ---- */
/* Principal branch of the Lambert W function. */
double frg_lambertw0(double z);
/* Estimated fraction of all roots collected, s W(-e^{-1/s}/s) + 1 with
 * s = successes / (successes + duplicates). */
double frg_estimate_collected(int64_t successes, int64_t duplicates);

#ifdef __cplusplus
}
#endif

#endif /* FRG_GB300_H */
