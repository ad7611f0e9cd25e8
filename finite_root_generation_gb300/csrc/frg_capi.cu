// C ABI of the tracker: contexts, configuration and the tracking entry points
// (include/frg_gb300.h). Replaces the reference driver's allocation block,
// InitRandStates/Homotopy launches and copies back (frg.cu:201-236, :351-404).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/frg_gb300.h"
#include <cuda_bf16.h>

#include "frg_kernels.h"
#include "frg_rng.h"

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

}  // namespace

namespace {
// Buffers of one round in flight: a round's launches use only its slot, so rounds on
// different slots (different streams) run concurrently.
struct Slot {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DevBuf gamma, gamma_lo, gamma_df, fpm_lo, fpm_df, task_start, queue, counters, starts;
  DevBuf handoff, handoff_list, lo_lists;
  DevBuf roots, codes, resid;  // staging of host outputs (frg_track_rounds)
  void release() {
    for (DevBuf* b : {&gamma, &gamma_lo, &gamma_df, &fpm_lo, &fpm_df, &task_start, &queue, &counters, &starts,
                      &handoff, &handoff_list, &lo_lists, &roots, &codes, &resid})
      b->release();
    if (own_stream && stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};
}  // namespace

struct frg_ctx {
  int device = 0;
  frg_config cfg;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int sm_count = 0;
  int blocks_per_sm[3] = {0, 0, 0};  // resident blocks per SM of each thread-per-path kernel mode
  int team_blocks_per_sm[4] = {0, 0, 0, 0};
  std::string err;
  DevBuf fpm, roots, codes, yfinal, resid;
  std::vector<Slot*> slots;           // slot 0 runs on `stream`
  std::vector<cudaEvent_t> round_ev;  // events around the mixed-precision launches of frg_track
  int last_rounds = 0;
  unsigned long long* h_counters = nullptr;  // pinned per-round counter copies (frg_track_rounds)
  size_t h_counters_n = 0;
  // call-wide buffers of frg_track_rounds with carry_handback: every round's task sets,
  // gammas and seeds, one hand-off record per path of the call, output staging
  DevBuf c_fpm, c_fpm_lo, c_fpm_df, c_gamma, c_gamma_lo, c_gamma_df, c_seeds, c_task_start, c_rec, c_roots,
      c_codes, c_resid;
  // early-retirement network (frg_set_mlp) and checkpoint features (frg_track_features)
  DevBuf mlp_w, mlp_norm, feat, nfeat;
  float mlp_threshold = 1.f;
  int mlp_every = 0;
  bool mlp_on = false;
  int feat_max = 0, feat_every = 0;
  bool feat_on = false;
};

static frg_status fail(frg_ctx* ctx, frg_status s, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return s;
}

static frg_status cuda_fail(frg_ctx* ctx, cudaError_t e, const char* where) {
  return fail(ctx, FRG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define FRG_CUDA(ctx, call)                                  \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

extern "C" frg_status frg_config_default(frg_config* c) {
  if (!c) return FRG_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  // htpytrack.cu:9-31
  c->s_init = 1.0; c->s_max = 100.0; c->s_min = 1e-6; c->rk_tol = 1e-3;
  c->caution_steps = 2;
  c->newt_its = 10; c->newt_tol = 1e-8; c->newt_residual = 1; c->newt_attempts = 3;
  c->sharp_its = 30; c->sharp_tol = 1e-12; c->sharp_residual = 1; c->sharp_attempts = 3;
  c->sharp_trigger = 1e-5; c->nudge_trigger = 1e-5;
  c->max_steps = 2000; c->max_ministeps = 3000;
  c->patch_range = 2.0;
  // frgkinematics.cu:7-8
  c->start_dist = FRG_START_UNIFORM; c->start_range = 5.0;
  // frg.cu:41
  c->gamma_mode = FRG_GAMMA_FIXED; c->gamma_re = 0.39231132891081666; c->gamma_im = 1.0062265257923928;
  // frgsupport.cu:7
  c->dup_tol = 1e-6;
  c->precision = FRG_PREC_FP64;
  c->t_switch = 0.99;
  c->cond_switch = 1e5;
  c->inf_tol = 0.0;
  c->threads_per_block = 0;
  c->blocks_per_sm = 0;
  c->newt_tol_lo = 1e-5;
  c->kernel_variant = FRG_KERNEL_TEAM;
  c->mixed_rounds = 1;
  c->lo_refine = 1;
  c->lo_endgame = 0;
  c->path_offset = 0;
  c->fp64_budget = 0;
  c->lo_points = 0;
  c->fp64_segment = 96;
  c->handback_good = 16;
  c->lo_final = 0;
  c->carry_handback = 0;
  c->round_graph = 0;
  c->system = 0;
  return FRG_OK;
}

frg_status frg_check_config(frg_ctx* ctx, const frg_config* c) {
  if (!c) return fail(ctx, FRG_ERR_ARG, "config is NULL");
  if (!(c->s_init > 0) || !(c->s_min > 0) || !(c->s_max >= c->s_min) || !(c->rk_tol > 0))
    return fail(ctx, FRG_ERR_ARG, "step sizes and rk_tol must be positive with s_max >= s_min");
  if (c->newt_its < 0 || c->sharp_its < 0 || c->newt_attempts < 1 || c->sharp_attempts < 1 ||
      c->max_steps < 0 || c->max_ministeps < 0)
    return fail(ctx, FRG_ERR_ARG, "iteration limits must be non-negative (attempts >= 1)");
  if (c->start_dist != FRG_START_UNIFORM && c->start_dist != FRG_START_NORMAL)
    return fail(ctx, FRG_ERR_ARG, "unknown start_dist");
  if (c->gamma_mode != FRG_GAMMA_FIXED && c->gamma_mode != FRG_GAMMA_RANDOM)
    return fail(ctx, FRG_ERR_ARG, "unknown gamma_mode");
  if (c->precision != FRG_PREC_FP64 && c->precision != FRG_PREC_MIXED)
    return fail(ctx, FRG_ERR_ARG, "unknown precision");
  if (c->kernel_variant != FRG_KERNEL_TEAM && c->kernel_variant != FRG_KERNEL_THREAD)
    return fail(ctx, FRG_ERR_ARG, "unknown kernel_variant");
  if (c->mixed_rounds < 0 || c->mixed_rounds > 64) return fail(ctx, FRG_ERR_ARG, "mixed_rounds must be in 0..64");
  if (c->path_offset < 0) return fail(ctx, FRG_ERR_ARG, "path_offset must be non-negative");
  if (c->fp64_budget < 0) return fail(ctx, FRG_ERR_ARG, "fp64_budget must be non-negative");
  if (c->lo_refine < 0 || c->lo_refine > 3) return fail(ctx, FRG_ERR_ARG, "lo_refine must be 0, 1, 2 or 3");
  if (c->lo_points < 0 || c->lo_points > 1) return fail(ctx, FRG_ERR_ARG, "lo_points must be 0 or 1");
  if (c->lo_final < 0 || c->lo_final > 1) return fail(ctx, FRG_ERR_ARG, "lo_final must be 0 or 1");
  if (c->carry_handback < 0 || c->carry_handback > 1) return fail(ctx, FRG_ERR_ARG, "carry_handback must be 0 or 1");
  if (c->round_graph < 0 || c->round_graph > 1) return fail(ctx, FRG_ERR_ARG, "round_graph must be 0 or 1");
  if (c->fp64_segment < 0 || c->handback_good < 0)
    return fail(ctx, FRG_ERR_ARG, "fp64_segment and handback_good must be non-negative");
  if (c->precision == FRG_PREC_MIXED && !(c->newt_tol_lo > 0 && c->cond_switch > 1 && c->t_switch <= 1.0))
    return fail(ctx, FRG_ERR_ARG, "mixed precision needs newt_tol_lo > 0, cond_switch > 1, t_switch <= 1");
  if (c->system < 0 || c->system >= frg_num_systems()) return fail(ctx, FRG_ERR_ARG, "unknown system");
  if (c->system != 0 && c->kernel_variant != FRG_KERNEL_THREAD)
    return fail(ctx, FRG_ERR_ARG, "plug-in systems run on the thread kernel");
  return FRG_OK;
}

extern "C" int frg_num_systems(void) { return frg_system_count(); }

extern "C" frg_status frg_system_info(int system, frg_system_desc* desc) {
  const char* name = nullptr;
  int nv = 0, np = 0;
  if (!desc || !frg_system_dims(system, &name, &nv, &np)) return FRG_ERR_ARG;
  std::memset(desc, 0, sizeof(*desc));
  std::strncpy(desc->name, name, sizeof(desc->name) - 1);
  desc->nv = nv;
  desc->np = np;
  return FRG_OK;
}

// Unknowns and parameters of the configured system.
static void dims_of(const frg_config& c, int* nv, int* np) {
  const char* name;
  if (!frg_system_dims(c.system, &name, nv, np)) { *nv = FRG_NV; *np = FRG_NP; }
}

extern "C" frg_status frg_create(frg_ctx** out, const frg_config* cfg, int device) {
  if (!out) return FRG_ERR_ARG;
  *out = nullptr;
  frg_ctx* ctx = new (std::nothrow) frg_ctx();
  if (!ctx) return FRG_ERR_ALLOC;
  frg_config def;
  frg_config_default(&def);
  ctx->cfg = cfg ? *cfg : def;
  frg_status s = frg_check_config(nullptr, &ctx->cfg);
  if (s != FRG_OK) { delete ctx; return s; }
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  for (int m = 0; m < 3 && e == cudaSuccess; ++m) {
    e = frg_track_occupancy(m, &ctx->blocks_per_sm[m]);
    if (ctx->blocks_per_sm[m] < 1) ctx->blocks_per_sm[m] = 1;
    if (e == cudaSuccess) e = frg_team_occupancy(m, &ctx->team_blocks_per_sm[m]);
    if (ctx->team_blocks_per_sm[m] < 1) ctx->team_blocks_per_sm[m] = 1;
  }
  if (e == cudaSuccess) e = frg_team_occupancy(3, &ctx->team_blocks_per_sm[3]);
  if (ctx->team_blocks_per_sm[3] < 1) ctx->team_blocks_per_sm[3] = 1;
  if (e == cudaSuccess) {
    Slot* s0 = new (std::nothrow) Slot();
    if (!s0) e = cudaErrorMemoryAllocation;
    else { s0->stream = ctx->stream; ctx->slots.push_back(s0); }
  }
  if (e != cudaSuccess) {
    frg_destroy(ctx);
    return FRG_ERR_CUDA;
  }
  *out = ctx;
  return FRG_OK;
}

extern "C" void frg_destroy(frg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (Slot* sl : ctx->slots) {
    if (sl->stream) cudaStreamSynchronize(sl->stream);
    sl->release();
    delete sl;
  }
  for (DevBuf* b : {&ctx->fpm, &ctx->roots, &ctx->codes, &ctx->yfinal, &ctx->resid, &ctx->mlp_w, &ctx->mlp_norm,
                    &ctx->feat, &ctx->nfeat, &ctx->c_fpm, &ctx->c_fpm_lo, &ctx->c_fpm_df, &ctx->c_gamma,
                    &ctx->c_gamma_lo, &ctx->c_gamma_df, &ctx->c_seeds, &ctx->c_task_start, &ctx->c_rec, &ctx->c_roots,
                    &ctx->c_codes, &ctx->c_resid})
    b->release();
  if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (cudaEvent_t e : ctx->round_ev) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

extern "C" const char* frg_last_error(const frg_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

extern "C" frg_status frg_set_config(frg_ctx* ctx, const frg_config* cfg) {
  if (!ctx) return FRG_ERR_ARG;
  frg_status s = frg_check_config(ctx, cfg);
  if (s != FRG_OK) return s;
  ctx->cfg = *cfg;
  return FRG_OK;
}

static int mixed_rounds_of(const frg_config& c) {
  return c.kernel_variant == FRG_KERNEL_TEAM ? (c.mixed_rounds > 0 ? c.mixed_rounds : 1) : 1;
}

static frg_status ensure_events(frg_ctx* ctx, std::vector<cudaEvent_t>& v, size_t n) {
  while (v.size() < n) {
    cudaEvent_t ev;
    FRG_CUDA(ctx, cudaEventCreate(&ev));
    v.push_back(ev);
  }
  return FRG_OK;
}

// gamma of task k: the configured constant (frg.cu:41) or e^{i phi}, phi uniform,
// drawn from a stream of `seed` reserved for gammas.
static void task_gammas(const frg_config& c, uint64_t seed, int ntasks, std::vector<cx<double>>& g) {
  g.resize(ntasks);
  for (int k = 0; k < ntasks; ++k) {
    if (c.gamma_mode == FRG_GAMMA_FIXED) {
      g[k] = cx<double>(c.gamma_re, c.gamma_im);
    } else {
      double phi = 6.283185307179586 * frg_uniform01(seed, 0xFFFFFFFFFFFFFFFFull - (uint64_t)k, 0);
      g[k] = cx<double>(std::cos(phi), std::sin(phi));
    }
  }
}

// One round on a slot: gammas, start values, then the tracking launches, all on `st`.
// `evs` (2 * mixed rounds + 1 events, mixed precision only) bracket the FP32 and FP64
// launches. Device pointers only here.
static frg_status enqueue_track(frg_ctx* ctx, Slot& sl, const cx<double>* d_fpm, int ntasks, const int64_t* ppt,
                                uint64_t seed, cx<double>* d_roots, int32_t* d_codes, cx<double>* d_yfinal,
                                double* d_resid, int64_t N, cudaStream_t st, cudaEvent_t* evs) {
  const bool mixed = ctx->cfg.precision == FRG_PREC_MIXED;
  int nv, np;
  dims_of(ctx->cfg, &nv, &np);
  std::vector<cx<double>> g;
  task_gammas(ctx->cfg, seed, ntasks, g);
  std::vector<cx<float>> g_lo(ntasks);
  std::vector<cx<df>> g_df(ntasks);
  for (int k = 0; k < ntasks; ++k) {
    g_lo[k] = cx<float>(g[k]);
    g_df[k] = cx<df>(df(g[k].re), df(g[k].im));
  }
  std::vector<int64_t> starts(ntasks + 1, 0);
  for (int k = 0; k < ntasks; ++k) starts[k + 1] = starts[k] + ppt[k];
  FRG_CUDA(ctx, sl.gamma.ensure(sizeof(cx<double>) * ntasks));
  FRG_CUDA(ctx, sl.gamma_lo.ensure(sizeof(cx<float>) * ntasks));
  FRG_CUDA(ctx, sl.fpm_lo.ensure(sizeof(cx<float>) * np * ntasks));
  FRG_CUDA(ctx, sl.fpm_df.ensure(sizeof(cx<df>) * np * ntasks));
  FRG_CUDA(ctx, sl.gamma_df.ensure(sizeof(cx<df>) * ntasks));
  FRG_CUDA(ctx, sl.task_start.ensure(sizeof(int64_t) * (ntasks + 1)));
  FRG_CUDA(ctx, sl.queue.ensure(sizeof(unsigned long long) * 8));
  FRG_CUDA(ctx, sl.counters.ensure(sizeof(unsigned long long) * FRG_NCOUNTERS));
  // (host-to-device copies from pageable memory are staged before these calls return)
  FRG_CUDA(ctx, cudaMemcpyAsync(sl.gamma_df.p, g_df.data(), sizeof(cx<df>) * ntasks, cudaMemcpyHostToDevice, st));
  FRG_CUDA(ctx, cudaMemcpyAsync(sl.gamma.p, g.data(), sizeof(cx<double>) * ntasks, cudaMemcpyHostToDevice, st));
  FRG_CUDA(ctx, cudaMemcpyAsync(sl.gamma_lo.p, g_lo.data(), sizeof(cx<float>) * ntasks, cudaMemcpyHostToDevice, st));
  FRG_CUDA(ctx, cudaMemcpyAsync(sl.task_start.p, starts.data(), sizeof(int64_t) * (ntasks + 1),
                                cudaMemcpyHostToDevice, st));
  FRG_CUDA(ctx, cudaMemsetAsync(sl.queue.p, 0, sizeof(unsigned long long) * 8, st));
  FRG_CUDA(ctx, cudaMemsetAsync(sl.counters.p, 0, sizeof(unsigned long long) * FRG_NCOUNTERS, st));
  FRG_CUDA(ctx, frg_launch_to_float(d_fpm, (cx<float>*)sl.fpm_lo.p, np * ntasks, st));
  FRG_CUDA(ctx, frg_launch_to_df(d_fpm, (cx<df>*)sl.fpm_df.p, np * ntasks, st));

  frg::TrackArgs a;
  std::memset(&a, 0, sizeof(a));
  a.cfg = ctx->cfg;
  a.fpm = d_fpm;
  a.gamma = (const cx<double>*)sl.gamma.p;
  a.fpm_lo = (const cx<float>*)sl.fpm_lo.p;
  a.gamma_lo = (const cx<float>*)sl.gamma_lo.p;
  a.fpm_df = (const cx<df>*)sl.fpm_df.p;
  a.gamma_df = (const cx<df>*)sl.gamma_df.p;
  a.task_start = (const int64_t*)sl.task_start.p;
  a.ntasks = ntasks;
  a.npaths = N;
  a.seed = seed;
  unsigned long long* q = (unsigned long long*)sl.queue.p;
  a.queue = q;
  a.roots = d_roots;
  a.codes = d_codes;
  a.yfinal = d_yfinal;
  a.resid = d_resid;
  a.work = nullptr;
  a.counters = (unsigned long long*)sl.counters.p;
  if (ctx->feat_on) {
    a.feat = (float*)ctx->feat.p;
    a.nfeat = (int32_t*)ctx->nfeat.p;
    a.feat_max = ctx->feat_max;
    a.feat_every = ctx->feat_every;
    FRG_CUDA(ctx, cudaMemsetAsync(ctx->nfeat.p, 0, sizeof(int32_t) * (size_t)N, st));
  }
  if (ctx->mlp_on) {
    a.mlp.w = (const __nv_bfloat16*)ctx->mlp_w.p;
    a.mlp.mu = (const float*)ctx->mlp_norm.p;
    a.mlp.inv_sigma = (const float*)ctx->mlp_norm.p + FRG_MLP_IN;
    a.mlp.threshold = ctx->mlp_threshold;
    a.mlp.every = ctx->mlp_every;
    a.feat_every = ctx->mlp_every;
  }
  const bool team = ctx->cfg.kernel_variant == FRG_KERNEL_TEAM;
  if (team) {  // start values for every path, generated once up front
    FRG_CUDA(ctx, sl.starts.ensure(sizeof(cx<double>) * frg::FRG_START_STRIDE * (size_t)N));
    a.starts = (const cx<double>*)sl.starts.p;
    cudaError_t e = frg_launch_starts(a, (cx<double>*)sl.starts.p, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "start kernel launch");
  }
  // persistent grids: SMs x resident blocks, capped by the work (one path per thread
  // for the thread kernels, one per 8 lanes for the team kernels)
  int plugin_bps[3] = {0, 0, 0};  // a plug-in system's kernels have their own occupancy
  if (ctx->cfg.system != 0)
    for (int m = 0; m < (mixed ? 3 : 1); ++m)
      FRG_CUDA(ctx, frg_track_occupancy_system(ctx->cfg.system, m, &plugin_bps[m]));
  auto grid_for = [&](int mode, int64_t n) {
    int bps = ctx->cfg.blocks_per_sm > 0             ? ctx->cfg.blocks_per_sm
              : (ctx->cfg.system != 0 && mode < 3)  ? plugin_bps[mode]
                                                    : (team ? ctx->team_blocks_per_sm[mode] : ctx->blocks_per_sm[mode]);
    int64_t grid = (int64_t)ctx->sm_count * bps;
    int64_t per_block = team ? FRG_TEAM_THREADS / 8 : FRG_TRACK_THREADS;
    int64_t need = (n + per_block - 1) / per_block;
    if (grid > need) grid = need;
    return (int)(grid < 1 ? 1 : grid);
  };
  auto launch = [&](int mode, int grid) {
    return team ? frg_launch_team(mode, a, grid, st) : frg_launch_track(mode, a, grid, st);
  };
  if (!mixed) {
    cudaError_t e = launch(0, grid_for(0, N));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "track kernel launch (FP64)");
    return FRG_OK;
  }
  // Rounds of (FP32 kernel, FP64 kernel). The FP64 kernel hands paths that are well
  // conditioned again (and before t_switch) back to the next round's FP32 kernel; the
  // last round keeps every path in FP64 until it ends. Queue heads and counts live in
  // q: [0] FP32 queue, [1] FP64 queue, [2] FP64 list count, [3], [4] hand-back counts.
  FRG_CUDA(ctx, sl.handoff.ensure(sizeof(frg::Handoff) * (size_t)N));
  FRG_CUDA(ctx, sl.handoff_list.ensure(sizeof(int64_t) * (size_t)N));
  FRG_CUDA(ctx, sl.lo_lists.ensure(sizeof(int64_t) * 2 * (size_t)N));
  a.handoff = (frg::Handoff*)sl.handoff.p;
  a.handoff_list = (int64_t*)sl.handoff_list.p;
  a.handoff_count = q + 2;
  int64_t* lo = (int64_t*)sl.lo_lists.p;
  const int rounds = mixed_rounds_of(ctx->cfg);
  FRG_CUDA(ctx, cudaEventRecord(evs[0], st));
  for (int r = 0; r < rounds; ++r) {
    if (r > 0) FRG_CUDA(ctx, cudaMemsetAsync(q, 0, sizeof(unsigned long long) * 3, st));
    FRG_CUDA(ctx, cudaMemsetAsync(q + 3 + (r & 1), 0, sizeof(unsigned long long), st));
    a.queue = q;
    a.lo_list = r == 0 ? nullptr : lo + (size_t)((r - 1) & 1) * N;
    a.lo_count = r == 0 ? nullptr : q + 3 + ((r - 1) & 1);
    a.back_list = nullptr;
    a.back_count = nullptr;
    a.lo_keep_ill = (ctx->cfg.lo_final && rounds > 1 && r + 1 == rounds) ? 1 : 0;
    const int lo_mode = (team && ctx->cfg.lo_points == 1) ? 3 : 1;
    cudaError_t e = launch(lo_mode, grid_for(lo_mode, N));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "track kernel launch (FP32 stage)");
    FRG_CUDA(ctx, cudaEventRecord(evs[2 * r + 1], st));
    a.queue = q + 1;
    a.lo_list = nullptr;
    a.lo_count = nullptr;
    a.back_list = (team && r + 1 < rounds) ? lo + (size_t)(r & 1) * N : nullptr;
    a.back_count = q + 3 + (r & 1);
    e = launch(2, grid_for(2, N));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "track kernel launch (FP64 stage)");
    FRG_CUDA(ctx, cudaEventRecord(evs[2 * r + 2], st));
  }
  return FRG_OK;
}

static frg_status check_track_args(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* ppt, double* roots,
                                   int32_t* codes, int64_t* N) {
  if (!ctx) return FRG_ERR_ARG;
  if (ntasks < 1 || !ppt || !fpm) return fail(ctx, FRG_ERR_ARG, "need ntasks >= 1, fpm and paths_per_task");
  int64_t n = 0;
  for (int k = 0; k < ntasks; ++k) {
    if (ppt[k] < 0) return fail(ctx, FRG_ERR_ARG, "paths_per_task must be non-negative");
    n += ppt[k];
  }
  if (n > 0 && (!roots || !codes)) return fail(ctx, FRG_ERR_ARG, "roots and codes are required");
  *N = n;
  return FRG_OK;
}

extern "C" frg_status frg_track_async(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                                      uint64_t seed, double* roots, int32_t* codes, double* yfinal, double* resid,
                                      void* stream) {
  int64_t N = 0;
  frg_status s = check_track_args(ctx, fpm, ntasks, paths_per_task, roots, codes, &N);
  if (s != FRG_OK) return s;
  if (N == 0) return FRG_OK;
  FRG_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!is_device_ptr(fpm) || !is_device_ptr(roots) || !is_device_ptr(codes) || (yfinal && !is_device_ptr(yfinal)) ||
      (resid && !is_device_ptr(resid)))
    return fail(ctx, FRG_ERR_ARG, "frg_track_async takes device pointers only");
  s = ensure_events(ctx, ctx->round_ev, 2 * mixed_rounds_of(ctx->cfg) + 1);
  if (s != FRG_OK) return s;
  ctx->last_rounds = 0;  // stage times are not reported for asynchronous calls
  return enqueue_track(ctx, *ctx->slots[0], (const cx<double>*)fpm, ntasks, paths_per_task, seed,
                       (cx<double>*)roots, codes, (cx<double>*)yfinal, resid, N, (cudaStream_t)stream,
                       ctx->round_ev.data());
}

// Adds one round's counters to stats (stats->paths and times are set by the caller).
static void add_counters(frg_stats* st, const unsigned long long* cnt, bool mixed) {
  for (int k = 0; k < 8; ++k) st->codes[k] += (int64_t)cnt[k];
  st->retired += (int64_t)cnt[36];
  st->ivp_solves += (int64_t)cnt[8];
  st->newton_iters += (int64_t)cnt[9];
  st->steps += (int64_t)cnt[10];
  st->fp64_solves += (int64_t)cnt[11];
  st->handoffs += (int64_t)cnt[12];
  for (int r = 0; r < 6; ++r) st->handoff_reason[r] += (int64_t)cnt[16 + r];
  for (int r = 0; r < 12; ++r) st->kernel_cycles[r] += (int64_t)cnt[24 + r];
  if (mixed) {
    st->handbacks += (int64_t)cnt[13];
    for (int b = 0; b < 6; ++b) st->fp64_segment_hist[b] += (int64_t)cnt[40 + b];
    if ((int64_t)cnt[46] > st->fp64_segment_max) st->fp64_segment_max = (int64_t)cnt[46];
    st->refine_solves += (int64_t)cnt[22];
    st->refine_warp_steps += (int64_t)cnt[23];
    st->refine_cycles += (int64_t)cnt[37];
  }
}

// FP32-stage and FP64-stage times of one call-round from its launch events.
static void stage_times(const cudaEvent_t* evs, int rounds, float* m32, float* m64, double* per_round) {
  *m32 = *m64 = 0.f;
  for (int r = 0; r < rounds; ++r) {
    float m0 = 0.f, m1 = 0.f;
    cudaEventElapsedTime(&m0, evs[2 * r], evs[2 * r + 1]);
    cudaEventElapsedTime(&m1, evs[2 * r + 1], evs[2 * r + 2]);
    *m32 += m0;
    *m64 += m1;
    if (per_round && r < 16) { per_round[2 * r] = m0; per_round[2 * r + 1] = m1; }
  }
}

extern "C" frg_status frg_track(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                                uint64_t seed, double* roots, int32_t* codes, double* yfinal, double* resid,
                                frg_stats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  int64_t N = 0;
  frg_status s = check_track_args(ctx, fpm, ntasks, paths_per_task, roots, codes, &N);
  if (s != FRG_OK) return s;
  if (stats) { std::memset(stats, 0, sizeof(*stats)); stats->paths = N; }
  if (N == 0) return FRG_OK;
  FRG_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  Slot& sl = *ctx->slots[0];
  const bool mixed = ctx->cfg.precision == FRG_PREC_MIXED;
  const int mr = mixed_rounds_of(ctx->cfg);
  s = ensure_events(ctx, ctx->round_ev, 2 * mr + 1);
  if (s != FRG_OK) return s;

  // inputs
  int nv, np;
  dims_of(ctx->cfg, &nv, &np);
  const cx<double>* d_fpm = (const cx<double>*)fpm;
  if (!is_device_ptr(fpm)) {
    FRG_CUDA(ctx, ctx->fpm.ensure(sizeof(cx<double>) * np * ntasks));
    FRG_CUDA(ctx, cudaMemcpyAsync(ctx->fpm.p, fpm, sizeof(cx<double>) * np * ntasks, cudaMemcpyHostToDevice, st));
    d_fpm = (const cx<double>*)ctx->fpm.p;
  }
  // outputs: written in place when on the device, staged otherwise
  struct Out { void* user; DevBuf* buf; size_t bytes; void* dev; bool host; };
  Out outs[4] = {{roots, &ctx->roots, sizeof(cx<double>) * nv * (size_t)N, nullptr, false},
                 {codes, &ctx->codes, sizeof(int32_t) * (size_t)N, nullptr, false},
                 {yfinal, &ctx->yfinal, sizeof(cx<double>) * (nv + 2) * (size_t)N, nullptr, false},
                 {resid, &ctx->resid, sizeof(double) * (size_t)N, nullptr, false}};
  for (Out& o : outs) {
    if (!o.user) continue;
    if (is_device_ptr(o.user)) { o.dev = o.user; }
    else {
      FRG_CUDA(ctx, o.buf->ensure(o.bytes));
      o.dev = o.buf->p;
      o.host = true;
    }
  }
  FRG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  s = enqueue_track(ctx, sl, d_fpm, ntasks, paths_per_task, seed, (cx<double>*)outs[0].dev, (int32_t*)outs[1].dev,
                    (cx<double>*)outs[2].dev, (double*)outs[3].dev, N, st, ctx->round_ev.data());
  if (s != FRG_OK) return s;
  ctx->last_rounds = mixed ? mr : 0;
  FRG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  for (Out& o : outs)
    if (o.user && o.host) FRG_CUDA(ctx, cudaMemcpyAsync(o.user, o.dev, o.bytes, cudaMemcpyDeviceToHost, st));
  unsigned long long cnt[FRG_NCOUNTERS];
  FRG_CUDA(ctx, cudaMemcpyAsync(cnt, sl.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, st));
  FRG_CUDA(ctx, cudaStreamSynchronize(st));
  if (stats) {
    add_counters(stats, cnt, mixed);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats->track_ms = ms;
    if (mixed) {
      float m32, m64;
      stage_times(ctx->round_ev.data(), mr, &m32, &m64, stats->round_ms);
      stats->stage_ms[0] = m32;
      stats->stage_ms[1] = m64;
    } else {
      stats->stage_ms[1] = ms;
    }
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return FRG_OK;
}

// frg_track_rounds with carry_handback: round r runs on slot r % depth; its FP64 launch
// hands paths that are well conditioned again to the FP32 launch of round r + depth (the
// next round on the same stream), which takes them before its fresh paths. Paths are
// addressed by their global index r * N + i, so records, lists and outputs are call-wide;
// the last `depth` rounds' FP64 launches finish every path they hold. d_fpm holds one
// task set (shared) or nrounds sets; outputs are device buffers of nrounds * N paths.
// evs: per round (per + 1) events, then one more for the end of the uploads. With
// round_graph the rounds of all streams are captured into one CUDA graph (the streams
// fork from and join into slot 0's stream), launched once, and this function returns
// after it finished.
static frg_status enqueue_rounds_carry(frg_ctx* ctx, const cx<double>* d_fpm, bool per_round_tasks, int ntasks,
                                       const int64_t* ppt, int nrounds, const uint64_t* seeds, int depth, int64_t N,
                                       cx<double>* d_roots, int32_t* d_codes, double* d_resid,
                                       std::vector<cudaEvent_t>& evs, int per) {
  const size_t K = (size_t)nrounds, T = (size_t)ntasks, KN = K * (size_t)N;
  cudaStream_t st0 = ctx->slots[0]->stream;
  // every round's task set (replicated when shared) in FP64, FP32 and double-float
  FRG_CUDA(ctx, ctx->c_fpm.ensure(sizeof(cx<double>) * FRG_NP * T * K));
  FRG_CUDA(ctx, ctx->c_fpm_lo.ensure(sizeof(cx<float>) * FRG_NP * T * K));
  FRG_CUDA(ctx, ctx->c_fpm_df.ensure(sizeof(cx<df>) * FRG_NP * T * K));
  cx<double>* c_fpm = (cx<double>*)ctx->c_fpm.p;
  const size_t set_bytes = sizeof(cx<double>) * FRG_NP * T;
  if (per_round_tasks) {
    FRG_CUDA(ctx, cudaMemcpyAsync(c_fpm, d_fpm, set_bytes * K, cudaMemcpyDeviceToDevice, st0));
  } else {
    for (size_t r = 0; r < K; ++r)
      FRG_CUDA(ctx, cudaMemcpyAsync((char*)c_fpm + set_bytes * r, d_fpm, set_bytes, cudaMemcpyDeviceToDevice, st0));
  }
  FRG_CUDA(ctx, frg_launch_to_float(c_fpm, (cx<float>*)ctx->c_fpm_lo.p, (int)(FRG_NP * T * K), st0));
  FRG_CUDA(ctx, frg_launch_to_df(c_fpm, (cx<df>*)ctx->c_fpm_df.p, (int)(FRG_NP * T * K), st0));
  // gammas of every round (the same per-round draw as frg_track), seeds, path offsets
  std::vector<cx<double>> g_all(T * K);
  std::vector<cx<float>> g_lo(T * K);
  std::vector<cx<df>> g_df(T * K);
  for (size_t r = 0; r < K; ++r) {
    std::vector<cx<double>> g;
    task_gammas(ctx->cfg, seeds[r], ntasks, g);
    for (size_t k = 0; k < T; ++k) {
      g_all[r * T + k] = g[k];
      g_lo[r * T + k] = cx<float>(g[k]);
      g_df[r * T + k] = cx<df>(df(g[k].re), df(g[k].im));
    }
  }
  std::vector<int64_t> starts(T + 1, 0);
  for (size_t k = 0; k < T; ++k) starts[k + 1] = starts[k] + ppt[k];
  FRG_CUDA(ctx, ctx->c_gamma.ensure(sizeof(cx<double>) * T * K));
  FRG_CUDA(ctx, ctx->c_gamma_lo.ensure(sizeof(cx<float>) * T * K));
  FRG_CUDA(ctx, ctx->c_gamma_df.ensure(sizeof(cx<df>) * T * K));
  FRG_CUDA(ctx, ctx->c_seeds.ensure(sizeof(uint64_t) * K));
  FRG_CUDA(ctx, ctx->c_task_start.ensure(sizeof(int64_t) * (T + 1)));
  FRG_CUDA(ctx, ctx->c_rec.ensure(sizeof(frg::Handoff) * KN));
  // per-slot lists: [0] FP64 queue of a round, [1 + p] paths carried between the slot's
  // rounds (p alternates); each holds at most every path of the call
  for (int d = 0; d < depth; ++d) {
    Slot& sl = *ctx->slots[d];
    FRG_CUDA(ctx, sl.lo_lists.ensure(sizeof(int64_t) * 3 * KN));
    FRG_CUDA(ctx, sl.queue.ensure(sizeof(unsigned long long) * 8));
    FRG_CUDA(ctx, sl.counters.ensure(sizeof(unsigned long long) * FRG_NCOUNTERS));
    FRG_CUDA(ctx, sl.starts.ensure(sizeof(cx<double>) * frg::FRG_START_STRIDE * (size_t)N));
  }
  // synchronous uploads: the host vectors go out of scope when this function returns
  FRG_CUDA(ctx, cudaStreamSynchronize(st0));
  FRG_CUDA(ctx, cudaMemcpy(ctx->c_gamma.p, g_all.data(), sizeof(cx<double>) * T * K, cudaMemcpyHostToDevice));
  FRG_CUDA(ctx, cudaMemcpy(ctx->c_gamma_lo.p, g_lo.data(), sizeof(cx<float>) * T * K, cudaMemcpyHostToDevice));
  FRG_CUDA(ctx, cudaMemcpy(ctx->c_gamma_df.p, g_df.data(), sizeof(cx<df>) * T * K, cudaMemcpyHostToDevice));
  FRG_CUDA(ctx, cudaMemcpy(ctx->c_seeds.p, seeds, sizeof(uint64_t) * K, cudaMemcpyHostToDevice));
  FRG_CUDA(ctx, cudaMemcpy(ctx->c_task_start.p, starts.data(), sizeof(int64_t) * (T + 1), cudaMemcpyHostToDevice));
  cudaEvent_t ev_ready = evs.back();
  FRG_CUDA(ctx, cudaEventRecord(ev_ready, st0));
  for (int d = 1; d < depth; ++d) FRG_CUDA(ctx, cudaStreamWaitEvent(ctx->slots[d]->stream, ev_ready, 0));

  const bool graph = ctx->cfg.round_graph != 0;
  cudaGraph_t g_graph = nullptr;
  cudaGraphExec_t g_exec = nullptr;
  std::vector<cudaEvent_t> fj;  // fork and join events of the capture
  struct GraphGuard {
    cudaGraph_t& g;
    cudaGraphExec_t& x;
    std::vector<cudaEvent_t>& ev;
    ~GraphGuard() {
      if (x) cudaGraphExecDestroy(x);
      if (g) cudaGraphDestroy(g);
      for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
  } gguard{g_graph, g_exec, fj};
  if (graph) {
    frg_status fs = ensure_events(ctx, fj, (size_t)depth + 1);
    if (fs != FRG_OK) return fs;
    FRG_CUDA(ctx, cudaStreamBeginCapture(st0, cudaStreamCaptureModeRelaxed));
    FRG_CUDA(ctx, cudaEventRecord(fj[0], st0));
    for (int d = 1; d < depth; ++d) FRG_CUDA(ctx, cudaStreamWaitEvent(ctx->slots[d]->stream, fj[0], 0));
  }
  // timing events: event-record nodes when captured
  auto record = [&](cudaEvent_t ev, cudaStream_t st) {
    return graph ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal) : cudaEventRecord(ev, st);
  };

  frg::TrackArgs a;
  std::memset(&a, 0, sizeof(a));
  a.cfg = ctx->cfg;
  a.fpm = c_fpm;
  a.gamma = (const cx<double>*)ctx->c_gamma.p;
  a.fpm_lo = (const cx<float>*)ctx->c_fpm_lo.p;
  a.gamma_lo = (const cx<float>*)ctx->c_gamma_lo.p;
  a.fpm_df = (const cx<df>*)ctx->c_fpm_df.p;
  a.gamma_df = (const cx<df>*)ctx->c_gamma_df.p;
  a.task_start = (const int64_t*)ctx->c_task_start.p;
  a.ntasks = ntasks;
  a.npaths = N;
  a.seeds = (const uint64_t*)ctx->c_seeds.p;
  a.roots = d_roots;
  a.codes = d_codes;
  a.resid = d_resid;
  a.handoff = (frg::Handoff*)ctx->c_rec.p;
  auto grid_for = [&](int mode) {
    int bps = ctx->cfg.blocks_per_sm > 0 ? ctx->cfg.blocks_per_sm : ctx->team_blocks_per_sm[mode];
    int64_t grid = (int64_t)ctx->sm_count * bps;
    return (int)(grid < 1 ? 1 : grid);
  };
  const int lo_mode = ctx->cfg.lo_points == 1 ? 3 : 1;
  auto rounds = [&]() -> frg_status {
    for (int r = 0; r < nrounds; ++r) {
      Slot& sl = *ctx->slots[r % depth];
      cudaStream_t st = sl.stream;
      cudaEvent_t* rev = evs.data() + (size_t)r * (per + 1);
      int64_t* lists = (int64_t*)sl.lo_lists.p;
      unsigned long long* q = (unsigned long long*)sl.queue.p;
      const int pout = (r / depth) & 1, pin = pout ^ 1;
      const bool has_in = r >= depth;
      // queue heads and this round's FP64-list count; the carried-in count (written by
      // this slot's previous FP64 launch) is kept
      FRG_CUDA(ctx, cudaMemsetAsync(q, 0, sizeof(unsigned long long) * 3, st));
      FRG_CUDA(ctx, cudaMemsetAsync(q + 3 + pout, 0, sizeof(unsigned long long), st));
      if (!has_in) FRG_CUDA(ctx, cudaMemsetAsync(q + 3 + pin, 0, sizeof(unsigned long long), st));
      FRG_CUDA(ctx, cudaMemsetAsync(sl.counters.p, 0, sizeof(unsigned long long) * FRG_NCOUNTERS, st));
      a.seed = seeds[r];
      a.round_base = (int64_t)r * N;
      a.counters = (unsigned long long*)sl.counters.p;
      a.starts = (const cx<double>*)sl.starts.p;
      {  // start values of this round's fresh paths (task set r)
        frg::TrackArgs sa = a;
        sa.fpm = c_fpm + (size_t)r * FRG_NP * T;
        cudaError_t e = frg_launch_starts(sa, (cx<double>*)sl.starts.p, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "start kernel launch");
      }
      FRG_CUDA(ctx, record(rev[0], st));
      // FP32 stage: carried paths, then this round's fresh paths
      a.queue = q;
      a.carry = 1;
      a.lo_list = has_in ? lists + (size_t)(1 + pin) * KN : nullptr;
      a.lo_count = has_in ? q + 3 + pin : nullptr;
      a.handoff_list = lists;
      a.handoff_count = q + 2;
      a.back_list = nullptr;
      a.back_count = nullptr;
      a.lo_keep_ill = 0;
      cudaError_t e = frg_launch_team(lo_mode, a, grid_for(lo_mode), st);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "track kernel launch (FP32 stage)");
      FRG_CUDA(ctx, record(rev[1], st));
      // FP64 stage: hand well-conditioned paths to round r + depth, or finish them all
      a.queue = q + 1;
      a.carry = 0;
      a.lo_list = nullptr;
      a.lo_count = nullptr;
      a.back_list = (r + depth < nrounds) ? lists + (size_t)(1 + pout) * KN : nullptr;
      a.back_count = q + 3 + pout;
      e = frg_launch_team(2, a, grid_for(2), st);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "track kernel launch (FP64 stage)");
      FRG_CUDA(ctx, record(rev[2], st));
      FRG_CUDA(ctx, record(rev[per], st));
      FRG_CUDA(ctx, cudaMemcpyAsync(ctx->h_counters + (size_t)r * FRG_NCOUNTERS, sl.counters.p,
                                    sizeof(unsigned long long) * FRG_NCOUNTERS, cudaMemcpyDeviceToHost, st));
    }
    return FRG_OK;
  };
  frg_status rs = rounds();
  if (rs != FRG_OK) {
    if (graph) {  // leave capture mode; the partial graph is discarded
      cudaGraph_t partial = nullptr;
      cudaStreamEndCapture(st0, &partial);
      if (partial) cudaGraphDestroy(partial);
      cudaGetLastError();
    }
    return rs;
  }
  if (graph) {
    for (int d = 1; d < depth; ++d) {
      FRG_CUDA(ctx, cudaEventRecord(fj[d], ctx->slots[d]->stream));
      FRG_CUDA(ctx, cudaStreamWaitEvent(st0, fj[d], 0));
    }
    FRG_CUDA(ctx, cudaStreamEndCapture(st0, &g_graph));
    FRG_CUDA(ctx, cudaGraphInstantiate(&g_exec, g_graph, 0));
    FRG_CUDA(ctx, cudaGraphLaunch(g_exec, st0));
    FRG_CUDA(ctx, cudaStreamSynchronize(st0));
  }
  return FRG_OK;
}

extern "C" frg_status frg_track_rounds(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                                       int nrounds, const uint64_t* seeds, int per_round_tasks, int depth,
                                       double* roots, int32_t* codes, double* resid, frg_stats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  if (!ctx) return FRG_ERR_ARG;
  if (nrounds < 1 || !seeds) return fail(ctx, FRG_ERR_ARG, "need nrounds >= 1 and one seed per round");
  if (depth < 1 || depth > 8) return fail(ctx, FRG_ERR_ARG, "depth must be in 1..8");
  if (per_round_tasks != 0 && per_round_tasks != 1) return fail(ctx, FRG_ERR_ARG, "per_round_tasks must be 0 or 1");
  int64_t N = 0;
  frg_status s = check_track_args(ctx, fpm, ntasks, paths_per_task, roots, codes, &N);
  if (s != FRG_OK) return s;
  if (stats) { std::memset(stats, 0, sizeof(*stats)); stats->paths = N * nrounds; }
  if (N == 0) return FRG_OK;
  FRG_CUDA(ctx, cudaSetDevice(ctx->device));
  const bool mixed = ctx->cfg.precision == FRG_PREC_MIXED;
  const int mr = mixed_rounds_of(ctx->cfg);
  if (depth > nrounds) depth = nrounds;
  while ((int)ctx->slots.size() < depth) {
    Slot* sl = new (std::nothrow) Slot();
    if (!sl) return fail(ctx, FRG_ERR_ALLOC, "slot allocation");
    cudaError_t e = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete sl; return cuda_fail(ctx, e, "cudaStreamCreateWithFlags"); }
    sl->own_stream = true;
    ctx->slots.push_back(sl);
  }
  // the task parameters (one set, or one per round), once, before any round
  const size_t task_sets = per_round_tasks ? (size_t)nrounds : 1;
  int nv, np;
  dims_of(ctx->cfg, &nv, &np);
  const cx<double>* d_fpm = (const cx<double>*)fpm;
  if (!is_device_ptr(fpm)) {
    FRG_CUDA(ctx, ctx->fpm.ensure(sizeof(cx<double>) * np * ntasks * task_sets));
    FRG_CUDA(ctx, cudaMemcpy(ctx->fpm.p, fpm, sizeof(cx<double>) * np * ntasks * task_sets,
                             cudaMemcpyHostToDevice));
    d_fpm = (const cx<double>*)ctx->fpm.p;
  }
  const bool dev_out = is_device_ptr(roots);
  if (is_device_ptr(codes) != dev_out || (resid && is_device_ptr(resid) != dev_out))
    return fail(ctx, FRG_ERR_ARG, "roots, codes and resid must all be device or all be host buffers");
  // pinned copies of every round's counters
  const size_t ncnt = (size_t)nrounds * FRG_NCOUNTERS;
  if (ctx->h_counters_n < ncnt) {
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    ctx->h_counters = nullptr;
    ctx->h_counters_n = 0;
    FRG_CUDA(ctx, cudaHostAlloc((void**)&ctx->h_counters, sizeof(unsigned long long) * ncnt, cudaHostAllocDefault));
    ctx->h_counters_n = ncnt;
  }
  // events: start, per round its launch events and its end
  const int per = 2 * mr + 1;
  std::vector<cudaEvent_t> evs;
  s = ensure_events(ctx, evs, (size_t)nrounds * (per + 1) + 1);
  if (s != FRG_OK) return s;
  struct EvGuard {
    std::vector<cudaEvent_t>& v;
    ~EvGuard() { for (cudaEvent_t e : v) cudaEventDestroy(e); }
  } guard{evs};
  cudaEvent_t ev_start = evs.back();
  FRG_CUDA(ctx, cudaEventRecord(ev_start, ctx->slots[0]->stream));
  for (int d = 1; d < depth; ++d) FRG_CUDA(ctx, cudaStreamWaitEvent(ctx->slots[d]->stream, ev_start, 0));
  const size_t rb = sizeof(cx<double>) * nv * (size_t)N, cb = sizeof(int32_t) * (size_t)N,
               eb = sizeof(double) * (size_t)N;
  const bool carry = mixed && ctx->cfg.carry_handback && ctx->cfg.kernel_variant == FRG_KERNEL_TEAM && mr == 1;
  if (carry) {
    // outputs: the caller's device buffers, or call-wide staging copied back at the end
    // (a round's paths may finish in a later round's launches)
    cx<double>* d_roots = (cx<double>*)roots;
    int32_t* d_codes = codes;
    double* d_resid = resid;
    if (!dev_out) {
      FRG_CUDA(ctx, ctx->c_roots.ensure(rb * nrounds));
      FRG_CUDA(ctx, ctx->c_codes.ensure(cb * nrounds));
      d_roots = (cx<double>*)ctx->c_roots.p;
      d_codes = (int32_t*)ctx->c_codes.p;
      if (resid) { FRG_CUDA(ctx, ctx->c_resid.ensure(eb * nrounds)); d_resid = (double*)ctx->c_resid.p; }
    }
    std::vector<cudaEvent_t> cev;
    s = ensure_events(ctx, cev, 1);
    if (s != FRG_OK) return s;
    struct CevGuard {
      std::vector<cudaEvent_t>& v;
      ~CevGuard() { for (cudaEvent_t e : v) cudaEventDestroy(e); }
    } cguard{cev};
    std::vector<cudaEvent_t> evs_c(evs.begin(), evs.end() - 1);
    evs_c.push_back(cev[0]);
    s = enqueue_rounds_carry(ctx, d_fpm, per_round_tasks != 0, ntasks, paths_per_task, nrounds, seeds, depth, N,
                             d_roots, d_codes, d_resid, evs_c, per);
    for (int d = 0; d < depth; ++d) cudaStreamSynchronize(ctx->slots[d]->stream);
    if (s != FRG_OK) return s;
    FRG_CUDA(ctx, cudaGetLastError());
    if (!dev_out) {
      FRG_CUDA(ctx, cudaMemcpy(roots, d_roots, rb * nrounds, cudaMemcpyDeviceToHost));
      FRG_CUDA(ctx, cudaMemcpy(codes, d_codes, cb * nrounds, cudaMemcpyDeviceToHost));
      if (resid) FRG_CUDA(ctx, cudaMemcpy(resid, d_resid, eb * nrounds, cudaMemcpyDeviceToHost));
    }
  } else {
  // on a failure part-way, rounds already enqueued must finish before the caller's
  // buffers can be reused: drain every slot's stream, then report the first error
  auto enqueue_all = [&]() -> frg_status {
    for (int r = 0; r < nrounds; ++r) {
      Slot& sl = *ctx->slots[r % depth];
      cudaStream_t st = sl.stream;
      cx<double>* d_roots;
      int32_t* d_codes;
      double* d_resid = nullptr;
      if (dev_out) {
        d_roots = (cx<double>*)((char*)roots + rb * r);
        d_codes = (int32_t*)((char*)codes + cb * r);
        if (resid) d_resid = (double*)((char*)resid + eb * r);
      } else {
        FRG_CUDA(ctx, sl.roots.ensure(rb));
        FRG_CUDA(ctx, sl.codes.ensure(cb));
        d_roots = (cx<double>*)sl.roots.p;
        d_codes = (int32_t*)sl.codes.p;
        if (resid) { FRG_CUDA(ctx, sl.resid.ensure(eb)); d_resid = (double*)sl.resid.p; }
      }
      cudaEvent_t* rev = evs.data() + (size_t)r * (per + 1);
      const cx<double>* fpm_r = d_fpm + (per_round_tasks ? (size_t)r * np * ntasks : 0);
      s = enqueue_track(ctx, sl, fpm_r, ntasks, paths_per_task, seeds[r], d_roots, d_codes, nullptr, d_resid, N, st,
                        rev);
      if (s != FRG_OK) return s;
      FRG_CUDA(ctx, cudaEventRecord(rev[per], st));
      if (!dev_out) {  // host outputs: asynchronous when the caller's buffers are pinned
        FRG_CUDA(ctx, cudaMemcpyAsync((char*)roots + rb * r, d_roots, rb, cudaMemcpyDeviceToHost, st));
        FRG_CUDA(ctx, cudaMemcpyAsync((char*)codes + cb * r, d_codes, cb, cudaMemcpyDeviceToHost, st));
        if (resid) FRG_CUDA(ctx, cudaMemcpyAsync((char*)resid + eb * r, d_resid, eb, cudaMemcpyDeviceToHost, st));
      }
      FRG_CUDA(ctx, cudaMemcpyAsync(ctx->h_counters + (size_t)r * FRG_NCOUNTERS, sl.counters.p,
                                    sizeof(unsigned long long) * FRG_NCOUNTERS, cudaMemcpyDeviceToHost, st));
    }
    return FRG_OK;
  };
  s = enqueue_all();
  if (s != FRG_OK) {
    for (int d = 0; d < depth; ++d) cudaStreamSynchronize(ctx->slots[d]->stream);
    return s;
  }
  for (int d = 0; d < depth; ++d) FRG_CUDA(ctx, cudaStreamSynchronize(ctx->slots[d]->stream));
  }
  if (stats) {
    float span = 0.f;
    for (int r = 0; r < nrounds; ++r) {
      add_counters(stats, ctx->h_counters + (size_t)r * FRG_NCOUNTERS, mixed);
      cudaEvent_t* rev = evs.data() + (size_t)r * (per + 1);
      float end = 0.f;
      cudaEventElapsedTime(&end, ev_start, rev[per]);
      if (end > span) span = end;
      if (mixed) {
        float m32, m64;
        stage_times(rev, mr, &m32, &m64, nullptr);
        stats->stage_ms[0] += m32;
        stats->stage_ms[1] += m64;
        if (r < 16) { stats->round_ms[2 * r] = m32; stats->round_ms[2 * r + 1] = m64; }
      }
    }
    stats->track_ms = span;
    if (!mixed) stats->stage_ms[1] = span;
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return FRG_OK;
}

extern "C" frg_status frg_set_mlp(frg_ctx* ctx, const float* params, const float* mu, const float* inv_sigma,
                                  float threshold, int every) {
  if (!ctx) return FRG_ERR_ARG;
  if (!params) {
    ctx->mlp_on = false;
    return FRG_OK;
  }
  if (!mu || !inv_sigma || every < 1 || !(threshold > 0.f && threshold <= 1.f))
    return fail(ctx, FRG_ERR_ARG, "frg_set_mlp needs mu, inv_sigma, every >= 1 and 0 < threshold <= 1");
  if (ctx->cfg.kernel_variant != FRG_KERNEL_TEAM)
    return fail(ctx, FRG_ERR_ARG, "early retirement runs in the team kernels");
  FRG_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<__nv_bfloat16> w(FRG_MLP_NPARAM);
  for (int i = 0; i < FRG_MLP_NPARAM; ++i) w[i] = __float2bfloat16_rn(params[i]);
  std::vector<float> norm(2 * FRG_MLP_IN);
  for (int i = 0; i < FRG_MLP_IN; ++i) { norm[i] = mu[i]; norm[FRG_MLP_IN + i] = inv_sigma[i]; }
  FRG_CUDA(ctx, ctx->mlp_w.ensure(sizeof(__nv_bfloat16) * FRG_MLP_NPARAM));
  FRG_CUDA(ctx, ctx->mlp_norm.ensure(sizeof(float) * 2 * FRG_MLP_IN));
  FRG_CUDA(ctx, cudaMemcpy(ctx->mlp_w.p, w.data(), sizeof(__nv_bfloat16) * FRG_MLP_NPARAM, cudaMemcpyHostToDevice));
  FRG_CUDA(ctx, cudaMemcpy(ctx->mlp_norm.p, norm.data(), sizeof(float) * 2 * FRG_MLP_IN, cudaMemcpyHostToDevice));
  ctx->mlp_threshold = threshold;
  ctx->mlp_every = every;
  ctx->mlp_on = true;
  return FRG_OK;
}

extern "C" frg_status frg_track_features(frg_ctx* ctx, const double* fpm, int ntasks, const int64_t* paths_per_task,
                                         uint64_t seed, double* roots, int32_t* codes, double* resid,
                                         float* features, int32_t* nfeat, int max_checkpoints, int every,
                                         frg_stats* stats) {
  if (!ctx) return FRG_ERR_ARG;
  if (!features || !nfeat || max_checkpoints < 1 || every < 1)
    return fail(ctx, FRG_ERR_ARG, "frg_track_features needs features, nfeat, max_checkpoints >= 1, every >= 1");
  if (ctx->cfg.kernel_variant != FRG_KERNEL_TEAM)
    return fail(ctx, FRG_ERR_ARG, "checkpoint features come from the team kernels");
  int64_t N = 0;
  for (int k = 0; k < ntasks && paths_per_task; ++k) N += paths_per_task[k];
  if (N <= 0) return frg_track(ctx, fpm, ntasks, paths_per_task, seed, roots, codes, nullptr, resid, stats);
  FRG_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t fb = sizeof(float) * FRG_MLP_IN * (size_t)max_checkpoints * (size_t)N;
  FRG_CUDA(ctx, ctx->feat.ensure(fb));
  FRG_CUDA(ctx, ctx->nfeat.ensure(sizeof(int32_t) * (size_t)N));
  ctx->feat_on = true;
  ctx->feat_max = max_checkpoints;
  ctx->feat_every = every;
  frg_status s = frg_track(ctx, fpm, ntasks, paths_per_task, seed, roots, codes, nullptr, resid, stats);
  ctx->feat_on = false;
  if (s != FRG_OK) return s;
  FRG_CUDA(ctx, cudaMemcpy(nfeat, ctx->nfeat.p, sizeof(int32_t) * (size_t)N, cudaMemcpyDeviceToHost));
  FRG_CUDA(ctx, cudaMemcpy(features, ctx->feat.p, fb, cudaMemcpyDeviceToHost));
  return FRG_OK;
}

