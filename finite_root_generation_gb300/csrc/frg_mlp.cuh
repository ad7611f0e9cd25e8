// Early-retirement network: a 32 -> 64 -> 64 -> 3 multilayer perceptron (ReLU) that
// reads a path's tracking features at a checkpoint and scores three outcomes: 0 the
// path ends at a new finite root, 1 it fails or diverges (no finite root with a small
// residual), 2 it ends at a root another path also reaches. Weights are BF16, inputs
// are standardised with the training set's mean and scale, sums accumulate in FP32.
//
// Parameter block (FP32 master copy, also the layout of the gradient):
//   W1[64][32] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#define FRG_MLP_IN 32
#define FRG_MLP_H 64
#define FRG_MLP_OUT 3
#define FRG_MLP_W1 0
#define FRG_MLP_B1 (FRG_MLP_W1 + FRG_MLP_H * FRG_MLP_IN)
#define FRG_MLP_W2 (FRG_MLP_B1 + FRG_MLP_H)
#define FRG_MLP_B2 (FRG_MLP_W2 + FRG_MLP_H * FRG_MLP_H)
#define FRG_MLP_W3 (FRG_MLP_B2 + FRG_MLP_H)
#define FRG_MLP_B3 (FRG_MLP_W3 + FRG_MLP_OUT * FRG_MLP_H)
#define FRG_MLP_NPARAM (FRG_MLP_B3 + FRG_MLP_OUT)

namespace frg {

// What the tracking kernels read: BF16 weights, FP32 normalisation and threshold.
struct MlpDevice {
  const __nv_bfloat16* w;  // FRG_MLP_NPARAM values in the layout above
  const float* mu;         // FRG_MLP_IN
  const float* inv_sigma;  // FRG_MLP_IN
  float threshold;         // retire when P(fails) >= threshold
  int every;               // checkpoint every this many accepted steps
};

// Logits of one feature vector (already standardised), one thread.
__device__ __forceinline__ void mlp_logits(const __nv_bfloat16* w, const float* x, float* out) {
  float h1[FRG_MLP_H], h2[FRG_MLP_H];
#pragma unroll 4
  for (int i = 0; i < FRG_MLP_H; ++i) {
    float a = __bfloat162float(w[FRG_MLP_B1 + i]);
    for (int k = 0; k < FRG_MLP_IN; ++k) a = fmaf(__bfloat162float(w[FRG_MLP_W1 + i * FRG_MLP_IN + k]), x[k], a);
    h1[i] = a > 0.f ? a : 0.f;
  }
#pragma unroll 4
  for (int i = 0; i < FRG_MLP_H; ++i) {
    float a = __bfloat162float(w[FRG_MLP_B2 + i]);
    for (int k = 0; k < FRG_MLP_H; ++k) a = fmaf(__bfloat162float(w[FRG_MLP_W2 + i * FRG_MLP_H + k]), h1[k], a);
    h2[i] = a > 0.f ? a : 0.f;
  }
  for (int i = 0; i < FRG_MLP_OUT; ++i) {
    float a = __bfloat162float(w[FRG_MLP_B3 + i]);
    for (int k = 0; k < FRG_MLP_H; ++k) a = fmaf(__bfloat162float(w[FRG_MLP_W3 + i * FRG_MLP_H + k]), h2[k], a);
    out[i] = a;
  }
}

// Softmax probability of class c from logits.
__device__ __forceinline__ float mlp_prob(const float* z, int c) {
  const float m = fmaxf(z[0], fmaxf(z[1], z[2]));
  const float e0 = __expf(z[0] - m), e1 = __expf(z[1] - m), e2 = __expf(z[2] - m);
  const float ec = c == 0 ? e0 : (c == 1 ? e1 : e2);
  return ec / (e0 + e1 + e2);
}

}  // namespace frg
