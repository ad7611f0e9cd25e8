// frg_track_noalloc: plain FP64 tracking that allocates no device memory.
//
// Who needs it: callers that may not call cudaMalloc / cudaFree themselves or
// through this library -- code that runs inside a host framework which owns all
// device memory through its own pool and forbids outside allocations, and loops
// that cannot afford the implicit device-wide synchronisation cudaFree performs
// (it would stall every other stream on the GPU). Such callers allocate their
// inputs and outputs once, up front, and call this entry point per round.
//
// The tracking kernels need a little scratch beyond the caller's inputs and
// outputs: the work-queue head, the per-call counters, and one gamma and one
// path-range offset per task. Here that scratch lives in one file-scope
// `static __device__` array, FRG_NOALLOC_SCRATCH_BYTES in size, which every GPU that
// loads the library keeps until the process exits. It bounds a call to
// FRG_NOALLOC_MAX_TASKS tasks; larger calls are rejected with FRG_ERR_ARG.
//
// Host code must not use the array's name as a device address (in host code it is
// only a stand-in). The first call on each device, with that device current, looks
// the address up once with cudaGetSymbolAddress and keeps it; make that first call
// before any stream capture. Every call shares the array and it keeps the previous
// call's contents, so each call first clears the queue head and counters; two calls
// whose GPU work overlaps (different streams on one device) race on the array.
//
// The per-task values (gammas, path counts) reach the array through a small set-up
// kernel that takes them as a launch parameter, so a call makes no host-to-device
// copy and reads no host memory after it returns.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/frg_gb300.h"
#include "frg_kernels.h"
#include "frg_rng.h"

namespace {

struct NoallocScratch {
  unsigned long long queue[4];
  unsigned long long counters[FRG_NCOUNTERS];
  cx<double> gamma[FRG_NOALLOC_MAX_TASKS];
  int64_t task_start[FRG_NOALLOC_MAX_TASKS + 1];
};
static_assert(sizeof(NoallocScratch) <= FRG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[FRG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up once per device).
frg_status scratch_on_current_device(NoallocScratch** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return FRG_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return FRG_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FRG_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<NoallocScratch*>(g_scratch_addr[dev]);
  return FRG_OK;
}

// Device (or managed) memory that the current device `dev` can use directly; device
// memory of another GPU is refused.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes attr;
  if (!p || cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (attr.type == cudaMemoryTypeManaged) return true;
  return attr.type == cudaMemoryTypeDevice && attr.device == dev;
}

// Per-task values of one call, passed by value as the set-up kernel's launch
// parameter (24.6 KB, inside the 32 KB parameter limit of this architecture).
struct NoallocTasks {
  int ntasks;
  int pad;
  cx<double> gamma[FRG_NOALLOC_MAX_TASKS];
  int64_t paths[FRG_NOALLOC_MAX_TASKS];
};
static_assert(sizeof(NoallocTasks) < 32000, "set-up parameters exceed the kernel parameter limit");

// One block: zero the queue head and counters, copy the gammas, prefix-sum the path
// counts into task_start.
__global__ void __launch_bounds__(256) noalloc_setup_kernel(NoallocScratch* sc, const __grid_constant__ NoallocTasks t) {
  for (int i = threadIdx.x; i < 4; i += blockDim.x) sc->queue[i] = 0ull;
  for (int i = threadIdx.x; i < FRG_NCOUNTERS; i += blockDim.x) sc->counters[i] = 0ull;
  for (int k = threadIdx.x; k < t.ntasks; k += blockDim.x) sc->gamma[k] = t.gamma[k];
  if (threadIdx.x == 0) {
    int64_t acc = 0;
    sc->task_start[0] = 0;
    for (int k = 0; k < t.ntasks; ++k) {
      acc += t.paths[k];
      sc->task_start[k + 1] = acc;
    }
  }
}

}  // namespace

extern "C" frg_status frg_track_noalloc(const frg_config* cfg, const double* fpm, int ntasks,
                                        const int64_t* paths_per_task, uint64_t seed, double* roots,
                                        int32_t* codes, double* resid, void* stream) {
  if (!cfg || !fpm || !paths_per_task || ntasks < 1) return FRG_ERR_ARG;
  if (ntasks > FRG_NOALLOC_MAX_TASKS) return FRG_ERR_ARG;  // beyond the static scratch
  // the same checks as frg_create / frg_set_config (step sizes, iteration limits,
  // modes), before any GPU work
  if (frg_check_config(nullptr, cfg) != FRG_OK) return FRG_ERR_ARG;
  if (cfg->precision != FRG_PREC_FP64) return FRG_ERR_ARG;  // mixed precision needs per-path buffers
  if (cfg->system != 0) return FRG_ERR_ARG;                 // its scratch holds Stephenson II tasks
  NoallocTasks tk;  // the set-up kernel's launch parameter, built on the host stack
  NoallocTasks* tp = &tk;
  tp->ntasks = ntasks;
  tp->pad = 0;
  int64_t N = 0;
  for (int k = 0; k < ntasks; ++k) {
    if (paths_per_task[k] < 0) return FRG_ERR_ARG;
    tp->paths[k] = paths_per_task[k];
    N += paths_per_task[k];
  }
  if (N == 0) return FRG_OK;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return FRG_ERR_CUDA;
  if (!roots || !codes || !on_device(fpm, dev) || !on_device(roots, dev) || !on_device(codes, dev) ||
      (resid && !on_device(resid, dev)))
    return FRG_ERR_ARG;  // inputs and outputs are the caller's buffers on the current device
  for (int k = 0; k < ntasks; ++k) {
    if (cfg->gamma_mode == FRG_GAMMA_FIXED) {
      tp->gamma[k] = cx<double>(cfg->gamma_re, cfg->gamma_im);
    } else {  // the same per-task draw as frg_track
      const double phi = 6.283185307179586 * frg_uniform01(seed, 0xFFFFFFFFFFFFFFFFull - (uint64_t)k, 0);
      tp->gamma[k] = cx<double>(std::cos(phi), std::sin(phi));
    }
  }
  NoallocScratch* sc = nullptr;
  frg_status s = scratch_on_current_device(&sc);
  if (s != FRG_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  // clear what must start at zero and fill the per-task values; the rest is overwritten
  noalloc_setup_kernel<<<1, 256, 0, st>>>(sc, *tp);
  if (cudaGetLastError() != cudaSuccess) return FRG_ERR_CUDA;

  frg::TrackArgs a;
  std::memset(&a, 0, sizeof(a));
  a.cfg = *cfg;
  a.fpm = (const cx<double>*)fpm;
  a.gamma = sc->gamma;
  a.task_start = sc->task_start;
  a.ntasks = ntasks;
  a.npaths = N;
  a.seed = seed;
  a.queue = sc->queue;
  a.roots = (cx<double>*)roots;
  a.codes = codes;
  a.resid = resid;
  a.counters = sc->counters;
  int sms = 0, bps = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return FRG_ERR_CUDA;
  const bool team = cfg->kernel_variant == FRG_KERNEL_TEAM;
  if ((team ? frg_team_occupancy(0, &bps) : frg_track_occupancy(0, &bps)) != cudaSuccess) return FRG_ERR_CUDA;
  if (cfg->blocks_per_sm > 0) bps = cfg->blocks_per_sm;
  if (bps < 1) bps = 1;
  const int64_t per_block = team ? FRG_TEAM_THREADS / 8 : FRG_TRACK_THREADS;
  int64_t grid = (int64_t)sms * bps, need = (N + per_block - 1) / per_block;
  if (grid > need) grid = need;
  const cudaError_t e = team ? frg_launch_team(0, a, (int)grid, st) : frg_launch_track(0, a, (int)grid, st);
  return e == cudaSuccess ? FRG_OK : FRG_ERR_CUDA;
}
