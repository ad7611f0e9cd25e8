// Device-resident root collection with duplicate marking (include/frg_gb300.h,
// frg_dcoll_*): the reference's SortingDeletingMerging (frgsupport.cu:10-215) with the
// driver's thrust ordering (frg.cu:432-435) done on the GPU, across rounds, for many
// tasks at once (one collection per key, e.g. per task).
//
// The duplicate rule is the host merge's (frg_collect.cpp), which restates the
// reference's: a success (code 0) becomes a duplicate (code 6) when every real
// component is within tol of a collected root of its key, or of a lower-index success
// of the same batch and key that is itself not a duplicate. Two roots within tol have
// Re(root[0]) in the same or adjacent cells of width 2 tol (the doubled width keeps that
// true after rounding x / (2 tol)), so candidates come from a hash table keyed by
// (key, cell) instead of the reference's sorted neighbour scan; every candidate is
// compared in all 42 components, so the marks are the same.
//
// One merge, all on the caller's stream:
//   1. check_coll     each success against the collection (read-only table)
//   2. insert_batch   the remaining successes into a batch table
//   3. check_batch    a success with no earlier in-batch match is kept; one with
//                     an earlier match is "dependent" (its status depends on the
//                     earlier roots' statuses)
//   4. resolve        one block walks the dependent roots in index order, the
//                     host rule applied sequentially (few roots: true duplicates)
//   5. append         kept roots join the collection and its table
// Roots whose first component is not finite never match (the host merge would let
// NaN compare equal); a success with a residual check has finite components. Every
// table probe is bounded by the table size.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <new>

#include "../../include/frg_gb300.h"

namespace {

constexpr int kReals = 2 * FRG_NV;
constexpr unsigned long long kEmpty = ~0ull;
constexpr int kThreads = 256;

struct DcollDev {
  double* roots;                  // capacity x 42
  int32_t* keys;                  // capacity collection keys
  unsigned long long* tkey;       // table: packed (key, cell) or kEmpty
  int64_t* tval;                  // table: root index
  unsigned long long tmask;       // table size - 1 (power of two)
  unsigned long long* size;       // [0] roots in the collection, [1] overflow flag
  int64_t capacity;
};

// (key, cell) packed into 64 bits: key in the top 20 bits, cell (clamped) in the low 44
__device__ __forceinline__ unsigned long long pack(int32_t key, long long cell) {
  const long long lim = (1ll << 43) - 1;
  cell = cell > lim ? lim : (cell < -lim ? -lim : cell);
  return ((unsigned long long)(uint32_t)key << 44) | ((unsigned long long)cell & ((1ull << 44) - 1));
}

__device__ __forceinline__ unsigned long long mix(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

// cell of width 2 tol of Re(root[0]); false if it is not finite
__device__ __forceinline__ bool cell_of(const double* r, double tol, long long* cell) {
  const double x = r[0];
  if (!(x - x == 0.0)) return false;
  *cell = (long long)floor(x * (0.5 / tol));
  return true;
}

// a success that takes part in the merge: code 0 and, when residuals are given, a
// residual of at most resid_max (a NaN residual fails)
__device__ __forceinline__ bool takes_part(const int32_t* codes, const double* resid, double resid_max, int64_t t) {
  return codes[t] == 0 && (!resid || resid[t] <= resid_max);
}

__device__ __forceinline__ bool same_root(const double* a, const double* b, double tol) {
  for (int k = 0; k < kReals; ++k)
    if (!(fabs(a[k] - b[k]) <= tol)) return false;
  return true;
}

__device__ void table_insert(unsigned long long* tkey, int64_t* tval, unsigned long long tmask,
                             unsigned long long k, int64_t v) {
  unsigned long long h = mix(k) & tmask;
  for (unsigned long long probe = 0; probe <= tmask; ++probe) {
    const unsigned long long prev = atomicCAS(&tkey[h], kEmpty, k);
    if (prev == kEmpty) {
      tval[h] = v;
      return;
    }
    h = (h + 1) & tmask;
  }
}

// 1. successes matching a collected root of their key become duplicates
__global__ void __launch_bounds__(kThreads) check_coll(DcollDev c, const double* roots, int32_t* codes,
                                                      const double* resid, double resid_max, const int32_t* keys,
                                                      int64_t n, double tol) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n || !takes_part(codes, resid, resid_max, t)) return;
  const double* rt = roots + (size_t)t * kReals;
  long long cell;
  if (!cell_of(rt, tol, &cell)) return;
  const int32_t key = keys ? keys[t] : 0;
  for (int dc = -1; dc <= 1; ++dc) {
    const unsigned long long k = pack(key, cell + dc);
    unsigned long long h = mix(k) & c.tmask;
    for (unsigned long long probe = 0; probe <= c.tmask; ++probe) {
      const unsigned long long e = c.tkey[h];
      if (e == kEmpty) break;
      if (e == k && same_root(rt, c.roots + (size_t)c.tval[h] * kReals, tol)) {
        codes[t] = FRG_CODE_DUPLICATE;
        return;
      }
      h = (h + 1) & c.tmask;
    }
  }
}

// 2. the remaining successes into the batch table
__global__ void __launch_bounds__(kThreads) insert_batch(const double* roots, const int32_t* codes,
                                                        const double* resid, double resid_max, const int32_t* keys,
                                                        int64_t n, double tol, unsigned long long* bkey,
                                                        int64_t* bval, unsigned long long bmask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n || !takes_part(codes, resid, resid_max, t)) return;
  long long cell;
  if (!cell_of(roots + (size_t)t * kReals, tol, &cell)) return;
  table_insert(bkey, bval, bmask, pack(keys ? keys[t] : 0, cell), t);
}

// 3. a success with an earlier matching success of the batch depends on it
__global__ void __launch_bounds__(kThreads) check_batch(const double* roots, const int32_t* codes,
                                                       const double* resid, double resid_max, const int32_t* keys,
                                                       int64_t n, double tol, const unsigned long long* bkey,
                                                       const int64_t* bval, unsigned long long bmask,
                                                       unsigned char* dep) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  dep[t] = 0;
  if (!takes_part(codes, resid, resid_max, t)) return;
  const double* rt = roots + (size_t)t * kReals;
  long long cell;
  if (!cell_of(rt, tol, &cell)) return;
  const int32_t key = keys ? keys[t] : 0;
  for (int dc = -1; dc <= 1; ++dc) {
    const unsigned long long k = pack(key, cell + dc);
    unsigned long long h = mix(k) & bmask;
    for (unsigned long long probe = 0; probe <= bmask; ++probe) {
      const unsigned long long e = bkey[h];
      if (e == kEmpty) break;
      const int64_t u = bval[h];
      if (e == k && u < t && same_root(rt, roots + (size_t)u * kReals, tol)) {
        dep[t] = 1;
        return;
      }
      h = (h + 1) & bmask;
    }
  }
}

// 4. dependent roots in index order: a duplicate when an earlier matching success is
//    still a success (the host merge's sequential rule). One block: the flags of each
//    chunk of 1,024 roots are compacted in order into shared memory, then thread 0
//    resolves them.
__global__ void __launch_bounds__(1024) resolve(const double* roots, int32_t* codes, const int32_t* keys, int64_t n,
                                                double tol, const unsigned long long* bkey, const int64_t* bval,
                                                unsigned long long bmask, const unsigned char* dep) {
  __shared__ int64_t list[1024];
  __shared__ int count;
  __shared__ int warp_base[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t t = base + threadIdx.x;
    const bool d = t < n && dep[t];
    const unsigned bal = __ballot_sync(0xffffffffu, d);
    if (lane == 0) warp_base[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int w = 0; w < 32; ++w) {
        const int cw = warp_base[w];
        warp_base[w] = acc;
        acc += cw;
      }
      count = acc;
    }
    __syncthreads();
    if (d) list[warp_base[warp] + __popc(bal & ((1u << lane) - 1))] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < count; ++i) {
        const int64_t tt = list[i];
        const double* rt = roots + (size_t)tt * kReals;
        long long cell = 0;
        cell_of(rt, tol, &cell);
        const int32_t key = keys ? keys[tt] : 0;
        bool dup = false;
        for (int dc = -1; dc <= 1 && !dup; ++dc) {
          const unsigned long long k = pack(key, cell + dc);
          unsigned long long h = mix(k) & bmask;
          for (unsigned long long probe = 0; probe <= bmask; ++probe) {
            const unsigned long long e = bkey[h];
            if (e == kEmpty) break;
            const int64_t u = bval[h];
            if (e == k && u < tt && codes[u] == 0 && same_root(rt, roots + (size_t)u * kReals, tol)) {
              dup = true;
              break;
            }
            h = (h + 1) & bmask;
          }
        }
        if (dup) codes[tt] = FRG_CODE_DUPLICATE;
      }
    }
    __syncthreads();
  }
}

// 5. kept successes join the collection
__global__ void __launch_bounds__(kThreads) append(DcollDev c, const double* roots, const int32_t* codes,
                                                  const double* resid, double resid_max, const int32_t* keys,
                                                  int64_t n, double tol) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n || !takes_part(codes, resid, resid_max, t)) return;
  const double* rt = roots + (size_t)t * kReals;
  const unsigned long long slot = atomicAdd(&c.size[0], 1ull);
  if ((int64_t)slot >= c.capacity) {
    c.size[1] = 1;  // overflow: the root is not collected
    return;
  }
  for (int k = 0; k < kReals; ++k) c.roots[slot * kReals + k] = rt[k];
  const int32_t key = keys ? keys[t] : 0;
  c.keys[slot] = key;
  long long cell;
  if (cell_of(rt, tol, &cell)) table_insert(c.tkey, c.tval, c.tmask, pack(key, cell), (int64_t)slot);
}

unsigned long long pow2_at_least(unsigned long long x) {
  unsigned long long p = 1024;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace

struct frg_dcoll {
  int device = 0;
  double tol = 1e-6;
  DcollDev d{};
  // batch scratch (grown on demand)
  unsigned long long* bkey = nullptr;
  int64_t* bval = nullptr;
  unsigned char* dep = nullptr;
  unsigned long long bsize = 0;
  int64_t bn = 0;
  unsigned long long* h_size = nullptr;  // pinned copy of d.size
};

static void dcoll_free_batch(frg_dcoll* c) {
  cudaFree(c->bkey);
  cudaFree(c->bval);
  cudaFree(c->dep);
  c->bkey = nullptr;
  c->bval = nullptr;
  c->dep = nullptr;
  c->bsize = 0;
  c->bn = 0;
}

extern "C" void frg_dcoll_destroy(frg_dcoll* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaDeviceSynchronize();
  cudaFree(c->d.roots);
  cudaFree(c->d.keys);
  cudaFree(c->d.tkey);
  cudaFree(c->d.tval);
  cudaFree(c->d.size);
  dcoll_free_batch(c);
  if (c->h_size) cudaFreeHost(c->h_size);
  delete c;
}

extern "C" frg_status frg_dcoll_create(frg_dcoll** out, int device, int64_t capacity, double dup_tol) {
  if (!out) return FRG_ERR_ARG;
  *out = nullptr;
  if (capacity < 1 || !(dup_tol > 0) || !std::isfinite(dup_tol)) return FRG_ERR_ARG;
  frg_dcoll* c = new (std::nothrow) frg_dcoll();
  if (!c) return FRG_ERR_ALLOC;
  c->device = device;
  c->tol = dup_tol;
  c->d.capacity = capacity;
  const unsigned long long tsize = pow2_at_least((unsigned long long)capacity * 2);
  c->d.tmask = tsize - 1;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaMalloc(&c->d.roots, sizeof(double) * kReals * (size_t)capacity);
  if (e == cudaSuccess) e = cudaMalloc(&c->d.keys, sizeof(int32_t) * (size_t)capacity);
  if (e == cudaSuccess) e = cudaMalloc(&c->d.tkey, sizeof(unsigned long long) * tsize);
  if (e == cudaSuccess) e = cudaMalloc(&c->d.tval, sizeof(int64_t) * tsize);
  if (e == cudaSuccess) e = cudaMalloc(&c->d.size, sizeof(unsigned long long) * 2);
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&c->h_size, sizeof(unsigned long long) * 2, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMemset(c->d.tkey, 0xff, sizeof(unsigned long long) * tsize);
  if (e == cudaSuccess) e = cudaMemset(c->d.size, 0, sizeof(unsigned long long) * 2);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    frg_dcoll_destroy(c);
    return FRG_ERR_CUDA;
  }
  *out = c;
  return FRG_OK;
}

extern "C" frg_status frg_dcoll_merge(frg_dcoll* c, const double* roots, int32_t* codes, const double* resid,
                                      double resid_max, const int32_t* keys, int64_t n, void* stream) {
  if (!c || n < 0 || (n > 0 && (!roots || !codes))) return FRG_ERR_ARG;
  if (n == 0) return FRG_OK;
  if (cudaSetDevice(c->device) != cudaSuccess) return FRG_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  if (n > c->bn) {
    if (cudaStreamSynchronize(st) != cudaSuccess) return FRG_ERR_CUDA;
    dcoll_free_batch(c);
    const unsigned long long bs = pow2_at_least((unsigned long long)n * 2);
    if (cudaMalloc(&c->bkey, sizeof(unsigned long long) * bs) != cudaSuccess ||
        cudaMalloc(&c->bval, sizeof(int64_t) * bs) != cudaSuccess || cudaMalloc(&c->dep, (size_t)n) != cudaSuccess) {
      dcoll_free_batch(c);
      return FRG_ERR_ALLOC;
    }
    c->bsize = bs;
    c->bn = n;
  }
  const unsigned long long bmask = c->bsize - 1;
  if (cudaMemsetAsync(c->bkey, 0xff, sizeof(unsigned long long) * c->bsize, st) != cudaSuccess) return FRG_ERR_CUDA;
  const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
  check_coll<<<grid, kThreads, 0, st>>>(c->d, roots, codes, resid, resid_max, keys, n, c->tol);
  insert_batch<<<grid, kThreads, 0, st>>>(roots, codes, resid, resid_max, keys, n, c->tol, c->bkey, c->bval, bmask);
  check_batch<<<grid, kThreads, 0, st>>>(roots, codes, resid, resid_max, keys, n, c->tol, c->bkey, c->bval, bmask,
                                         c->dep);
  resolve<<<1, 1024, 0, st>>>(roots, codes, keys, n, c->tol, c->bkey, c->bval, bmask, c->dep);
  append<<<grid, kThreads, 0, st>>>(c->d, roots, codes, resid, resid_max, keys, n, c->tol);
  return cudaGetLastError() == cudaSuccess ? FRG_OK : FRG_ERR_CUDA;
}

extern "C" frg_status frg_dcoll_size(frg_dcoll* c, void* stream, int64_t* size) {
  if (!c || !size) return FRG_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return FRG_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(c->h_size, c->d.size, sizeof(unsigned long long) * 2, cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return FRG_ERR_CUDA;
  if (c->h_size[1]) return FRG_ERR_ALLOC;  // a merge ran out of capacity
  *size = (int64_t)c->h_size[0];
  return FRG_OK;
}

extern "C" frg_status frg_dcoll_get(frg_dcoll* c, double* roots, int32_t* keys, int64_t capacity) {
  if (!c) return FRG_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return FRG_ERR_CUDA;
  int64_t n = 0;
  frg_status s = frg_dcoll_size(c, nullptr, &n);
  if (s != FRG_OK) return s;
  if (capacity < n || (n > 0 && !roots)) return FRG_ERR_ARG;
  if (n == 0) return FRG_OK;
  if (cudaMemcpy(roots, c->d.roots, sizeof(double) * kReals * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return FRG_ERR_CUDA;
  if (keys && cudaMemcpy(keys, c->d.keys, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return FRG_ERR_CUDA;
  return FRG_OK;
}
