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

#include "../../finite_root_generation_gb300/csrc/frg_rng.h"

typedef struct {
  unsigned long long seed;
  unsigned long long stream;
  unsigned long long index;
} curandState;

static inline void curand_init(unsigned long long seed, unsigned long long subsequence,
                               unsigned long long offset, curandState* state) {
  state->seed = seed;
  state->stream = subsequence;
  state->index = offset;
}

static inline double curand_uniform_double(curandState* state) {
  return frg_uniform01(state->seed, state->stream, state->index++);
}

#endif
