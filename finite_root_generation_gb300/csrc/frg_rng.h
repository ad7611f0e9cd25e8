/*
 * Counter-based random numbers for the path tracker: Philox4x32-10.
 *
 * Written from the published description of Philox (J. K. Salmon, M. A. Moraes,
 * R. O. Dror, D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11):
 * ten rounds of two 32x32->64 multiplies with a Weyl key schedule.
 *
 * Every random draw of a path is a pure function of (seed, stream, index):
 *   block = index >> 1, counter = {block.lo, block.hi, stream.lo, stream.hi},
 *   key = {seed.lo, seed.hi}; an even index takes output words 0,1 and an odd
 *   index takes words 2,3; the 53-bit double is (w_a >> 5) * 2^26 + (w_b >> 6),
 *   mapped to (0, 1] like curand_uniform_double.
 *
 * The reference draws its numbers from a per-thread curand XORWOW state
 * (frg.cu:30-33, frgkinematics.cu:41-58, htpytrack.cu:55-66). This stream replaces
 * it, so a path's draws do not depend on how paths are laid out on the device and
 * the host build of the reference (through a curand_kernel.h shim that calls these
 * functions) sees exactly the same numbers as the CUDA kernels.
 *
 * This header is plain C99 and also compiles as CUDA device code.
 */
#ifndef FRG_RNG_H
#define FRG_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define FRG_RNG_FN static __host__ __device__ __forceinline__
#else
#define FRG_RNG_FN static inline
#endif

#define FRG_PHILOX_M0 0xD2511F53u
#define FRG_PHILOX_M1 0xCD9E8D57u
#define FRG_PHILOX_W0 0x9E3779B9u
#define FRG_PHILOX_W1 0xBB67AE85u

/* One Philox4x32 block: 10 rounds, key bumped between rounds. */
FRG_RNG_FN void frg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)FRG_PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)FRG_PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += FRG_PHILOX_W0;
    k1 += FRG_PHILOX_W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Draw number `index` of stream `stream` under `seed`, uniform on (0, 1]. */
FRG_RNG_FN double frg_uniform01(uint64_t seed, uint64_t stream, uint64_t index) {
  uint64_t block = index >> 1;
  uint32_t ctr[4] = {(uint32_t)block, (uint32_t)(block >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t w[4];
  frg_philox4x32_10(ctr, key, w);
  uint32_t a = (index & 1) ? w[2] : w[0];
  uint32_t b = (index & 1) ? w[3] : w[1];
  uint64_t v = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)(v + 1) * (1.0 / 9007199254740992.0); /* 2^-53 */
}

#endif /* FRG_RNG_H */
