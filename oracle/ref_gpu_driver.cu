/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * GPU build of the reference tracker: the reference's own kernels InitRandStates and
 * Homotopy (frg.cu:30-124), with every device function they call, compiled unchanged
 * by nvcc -rdc=true for sm_103a (oracle/Makefile target refgpu), and launched by this
 * driver. The driver takes the place of the reference's main (frg.cu:128-553), which is
 * compiled under another name and never called, and differs from it only where main
 * would not run as a measurement: no argument parsing (frg.cu:132 reads argv[1] before
 * checking argc), the seed is a parameter instead of time(NULL) (:359), the grid covers
 * `npaths` (a multiple of the reference's 256 threads per block) instead of the
 * compile-time 80 x 256 (:25-27), and nothing dereferences device memory on the host
 * (:432): roots and codes come back with cudaMemcpy as at :389, :398.
 *
 * Two builds: librefgpu.so with the reference's curand XORWOW streams (curand_kernel.h
 * of the CUDA toolkit), and librefgpu_philox.so with oracle/ref_stub/curand_kernel.h,
 * whose Philox streams are the CUDA tracker's own, so the reference's GPU paths can be
 * compared with it path for path.
 */
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cstring>

#include "classes.cuh"
#include "htpykinematics.cuh"

__global__ void InitRandStates(curandState* randStates, unsigned long long seed);
__global__ void Homotopy(curandState* randStates, Vect<nP>* fpm, Vect<nV>* fpt, int* errorCodes,
                         Vect<nV + 2>* vectDebug, Matr<nV + 2, nV + 2>* matrDebug);

extern "C" {

/* Size of one path's RNG state in this build (curand XORWOW or the Philox stub). */
int refgpu_state_bytes(void) { return (int)sizeof(curandState); }

/* Track `npaths` paths (a positive multiple of 256) of the target `fpm` (30 complex) with
 * the reference's kernels: InitRandStates(seed) then Homotopy, 256 threads per block as
 * at frg.cu:26. Outputs: roots (npaths x 21 complex, canonical cognate), codes; ms[0] =
 * the two kernels, ms[1] = kernels + copies back (the span the reference times,
 * frg.cu:356, :422-426). Returns 0 or a cudaError_t value; err (optional) gets its name. */
int refgpu_track(const double* fpm, unsigned long long seed, long long npaths, double* roots, int* codes,
                 float* ms, char* err, int errlen) {
  const int threads = 256;
  if (npaths <= 0 || npaths % threads) return (int)cudaErrorInvalidValue;
  const long long blocks = npaths / threads;
  curandState* d_states = nullptr;
  Vect<nP>* d_fpm = nullptr;
  Vect<nV>* d_fpt = nullptr;
  int* d_codes = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  cudaError_t st = cudaSuccess;
  auto ok = [&](cudaError_t e) {
    if (st == cudaSuccess && e != cudaSuccess) st = e;
    return st == cudaSuccess;
  };
  if (ok(cudaMalloc(&d_states, sizeof(curandState) * npaths)) && ok(cudaMalloc(&d_fpm, sizeof(Vect<nP>))) &&
      ok(cudaMalloc(&d_fpt, sizeof(Vect<nV>) * npaths)) && ok(cudaMalloc(&d_codes, sizeof(int) * npaths)) &&
      ok(cudaEventCreate(&e0)) && ok(cudaEventCreate(&e1)) && ok(cudaEventCreate(&e2)) &&
      ok(cudaMemcpy(d_fpm, fpm, sizeof(Vect<nP>), cudaMemcpyHostToDevice)) && ok(cudaDeviceSynchronize())) {
    cudaEventRecord(e0);
    InitRandStates<<<(unsigned)blocks, threads>>>(d_states, seed);
    if (ok(cudaGetLastError())) {
      Homotopy<<<(unsigned)blocks, threads>>>(d_states, d_fpm, d_fpt, d_codes, nullptr, nullptr);
      if (ok(cudaGetLastError())) {
        cudaEventRecord(e1);
        if (ok(cudaMemcpy(roots, d_fpt, sizeof(Vect<nV>) * npaths, cudaMemcpyDeviceToHost)) &&
            ok(cudaMemcpy(codes, d_codes, sizeof(int) * npaths, cudaMemcpyDeviceToHost))) {
          cudaEventRecord(e2);
          if (ok(cudaEventSynchronize(e2))) {
            cudaEventElapsedTime(&ms[0], e0, e1);
            cudaEventElapsedTime(&ms[1], e0, e2);
          }
        }
      }
    }
  }
  if (st != cudaSuccess && err && errlen > 0) {
    std::strncpy(err, cudaGetErrorName(st), (size_t)errlen - 1);
    err[errlen - 1] = 0;
  }
  cudaFree(d_states);
  cudaFree(d_fpm);
  cudaFree(d_fpt);
  cudaFree(d_codes);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e2) cudaEventDestroy(e2);
  return (int)st;
}

}  // extern "C"
