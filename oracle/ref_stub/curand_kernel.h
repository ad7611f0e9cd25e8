/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * A stand-in for CUDA's curand_kernel.h, placed first on the include path when
 * the reference tracker's own sources are compiled for the host (oracle/Makefile).
 * It supplies only the three names the reference uses -- curandState,
 * curand_init (frg.cu:32) and curand_uniform_double (frgkinematics.cu:41-58,74,101;
 * htpytrack.cu:56-66,148-149,207-208) -- backed by the Philox stream of
 * frg_rng.h, so the host-built reference and the CUDA kernels draw identical
 * numbers for a path.
 *
 * The reference passes curandState BY VALUE into GenerateStart and TrackPath
 * (frgkinematics.cu:13, htpytrack.cu:33-34); with this state (seed, stream, next
 * index) that copy semantics is reproduced exactly.
 */
#ifndef FRG_ORACLE_CURAND_STUB_H
#define FRG_ORACLE_CURAND_STUB_H

#include <math.h>

#include "../../finite_root_generation_gb300/csrc/frg_rng.h"

/* host functions for the host build; host and device functions under nvcc (the GPU
   build of the reference's kernels, oracle/ref_gpu_driver.cu) */
#if defined(__CUDACC__)
#define FRG_STUB_FN static __host__ __device__ __forceinline__
#else
#define FRG_STUB_FN static inline
#endif

typedef struct {
  unsigned long long seed;
  unsigned long long stream;
  unsigned long long index;
  int mode; /* 0: the path's uniform draws in order; 1: complex-normal start values */
} curandState;

FRG_STUB_FN void curand_init(unsigned long long seed, unsigned long long subsequence,
                               unsigned long long offset, curandState* state) {
  state->seed = seed;
  state->stream = subsequence;
  state->index = offset;
  state->mode = 0;
}

/* Mode 1 serves GenerateStart (frgkinematics.cu:41-58) when the start mechanisms are
 * complex normal instead of the reference's U(-5,5)^2: its k-th draw of the 46 start
 * values is returned as (g + 5) / 10, so that GenerateStart's own map 10 u - 5 yields
 * g, a N(0, 1/2) component drawn by Box-Muller from draws 2k and 2k + 1 of the path's
 * stream (the tracking kernels' start_dist = 1 order); its later draws (the quadratic
 * branches, :74, :101) come from index 92 on. TrackPath receives a mode-0 copy. */
FRG_STUB_FN double curand_uniform_double(curandState* state) {
  if (state->mode == 1) {
    const unsigned long long k = state->index++;
    if (k < 46) {
      const double u1 = frg_uniform01(state->seed, state->stream, 2 * k);
      const double u2 = frg_uniform01(state->seed, state->stream, 2 * k + 1);
      const double g = sqrt(-log(u1)) * cos(6.283185307179586 * u2);
      return (g + 5.0) / 10.0;
    }
    return frg_uniform01(state->seed, state->stream, 92 + (k - 46));
  }
  return frg_uniform01(state->seed, state->stream, state->index++);
}

#endif
