// Training and batch inference of the early-retirement network (frg_mlp.cuh) with
// hand-written kernels: forward and backward per sample in one kernel (BF16 weights,
// FP32 sums, gradients reduced in shared memory and then across blocks), an Adam step,
// and a host loop over shuffled mini-batches. No counterpart in the reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/frg_gb300.h"
#include "frg_mlp.cuh"

namespace {

constexpr int kThreads = 128;

__global__ void to_bf16_kernel(const float* p, __nv_bfloat16* w, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = __float2bfloat16_rn(p[i]);
}

// Loss and gradient of a batch: sample b is X[idx[b]] (idx null: b itself). Mean over
// the batch of the class-weighted cross entropy; the gradient is with respect to the
// BF16 weights the forward pass used.
__global__ void __launch_bounds__(kThreads) grad_kernel(const float* X, const int32_t* y, const int64_t* idx,
                                                       int64_t B, const __nv_bfloat16* w, const float* class_w,
                                                       float* grad, double* loss) {
  __shared__ float g[FRG_MLP_NPARAM];
  __shared__ float sloss;
  for (int i = threadIdx.x; i < FRG_MLP_NPARAM; i += kThreads) g[i] = 0.f;
  if (threadIdx.x == 0) sloss = 0.f;
  __syncthreads();
  const int64_t b = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (b < B) {
    const int64_t s = idx ? idx[b] : b;
    float x[FRG_MLP_IN], h1[FRG_MLP_H], h2[FRG_MLP_H], z[FRG_MLP_OUT];
    for (int k = 0; k < FRG_MLP_IN; ++k) x[k] = X[s * FRG_MLP_IN + k];
    for (int i = 0; i < FRG_MLP_H; ++i) {
      float a = __bfloat162float(w[FRG_MLP_B1 + i]);
      for (int k = 0; k < FRG_MLP_IN; ++k) a = fmaf(__bfloat162float(w[FRG_MLP_W1 + i * FRG_MLP_IN + k]), x[k], a);
      h1[i] = a > 0.f ? a : 0.f;
    }
    for (int i = 0; i < FRG_MLP_H; ++i) {
      float a = __bfloat162float(w[FRG_MLP_B2 + i]);
      for (int k = 0; k < FRG_MLP_H; ++k) a = fmaf(__bfloat162float(w[FRG_MLP_W2 + i * FRG_MLP_H + k]), h1[k], a);
      h2[i] = a > 0.f ? a : 0.f;
    }
    for (int i = 0; i < FRG_MLP_OUT; ++i) {
      float a = __bfloat162float(w[FRG_MLP_B3 + i]);
      for (int k = 0; k < FRG_MLP_H; ++k) a = fmaf(__bfloat162float(w[FRG_MLP_W3 + i * FRG_MLP_H + k]), h2[k], a);
      z[i] = a;
    }
    const int c = y[s];
    const float m = fmaxf(z[0], fmaxf(z[1], z[2]));
    float e[FRG_MLP_OUT], se = 0.f;
    for (int i = 0; i < FRG_MLP_OUT; ++i) { e[i] = expf(z[i] - m); se += e[i]; }
    const float wc = class_w[c] / (float)B;
    atomicAdd(&sloss, -wc * (z[c] - m - logf(se)));
    // backward
    float dz[FRG_MLP_OUT];
    for (int i = 0; i < FRG_MLP_OUT; ++i) dz[i] = wc * (e[i] / se - (i == c ? 1.f : 0.f));
    float dh2[FRG_MLP_H];
    for (int k = 0; k < FRG_MLP_H; ++k) dh2[k] = 0.f;
    for (int i = 0; i < FRG_MLP_OUT; ++i) {
      atomicAdd(&g[FRG_MLP_B3 + i], dz[i]);
      for (int k = 0; k < FRG_MLP_H; ++k) {
        atomicAdd(&g[FRG_MLP_W3 + i * FRG_MLP_H + k], dz[i] * h2[k]);
        dh2[k] = fmaf(__bfloat162float(w[FRG_MLP_W3 + i * FRG_MLP_H + k]), dz[i], dh2[k]);
      }
    }
    float dh1[FRG_MLP_H];
    for (int k = 0; k < FRG_MLP_H; ++k) dh1[k] = 0.f;
    for (int i = 0; i < FRG_MLP_H; ++i) {
      if (h2[i] <= 0.f) continue;  // ReLU
      const float d = dh2[i];
      atomicAdd(&g[FRG_MLP_B2 + i], d);
      for (int k = 0; k < FRG_MLP_H; ++k) {
        if (h1[k] > 0.f) atomicAdd(&g[FRG_MLP_W2 + i * FRG_MLP_H + k], d * h1[k]);
        dh1[k] = fmaf(__bfloat162float(w[FRG_MLP_W2 + i * FRG_MLP_H + k]), d, dh1[k]);
      }
    }
    for (int i = 0; i < FRG_MLP_H; ++i) {
      if (h1[i] <= 0.f) continue;
      const float d = dh1[i];
      atomicAdd(&g[FRG_MLP_B1 + i], d);
      for (int k = 0; k < FRG_MLP_IN; ++k) atomicAdd(&g[FRG_MLP_W1 + i * FRG_MLP_IN + k], d * x[k]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < FRG_MLP_NPARAM; i += kThreads)
    if (g[i] != 0.f) atomicAdd(&grad[i], g[i]);
  if (threadIdx.x == 0) atomicAdd(loss, (double)sloss);
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

__global__ void predict_kernel(const float* X, int64_t n, const __nv_bfloat16* w, float* probs) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[FRG_MLP_IN], z[FRG_MLP_OUT];
  for (int k = 0; k < FRG_MLP_IN; ++k) x[k] = X[s * FRG_MLP_IN + k];
  frg::mlp_logits(w, x, z);
  for (int c = 0; c < FRG_MLP_OUT; ++c) probs[s * FRG_MLP_OUT + c] = frg::mlp_prob(z, c);
}

struct Dev {
  void* p = nullptr;
  ~Dev() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, n); }
};

#define MLP_CUDA(call)                          \
  do {                                          \
    if ((call) != cudaSuccess) return FRG_ERR_CUDA; \
  } while (0)

int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

extern "C" int frg_mlp_param_count(void) { return FRG_MLP_NPARAM; }

extern "C" frg_status frg_mlp_grad(const float* X, const int32_t* y, int64_t n, const float* params,
                                   const float* class_w, float* grad, double* loss) {
  if (!X || !y || n < 1 || !params || !class_w || !grad || !loss) return FRG_ERR_ARG;
  Dev dX, dy, dp, dw, dcw, dg, dl;
  MLP_CUDA(dX.alloc(sizeof(float) * FRG_MLP_IN * n));
  MLP_CUDA(dy.alloc(sizeof(int32_t) * n));
  MLP_CUDA(dp.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(dw.alloc(sizeof(__nv_bfloat16) * FRG_MLP_NPARAM));
  MLP_CUDA(dcw.alloc(sizeof(float) * FRG_MLP_OUT));
  MLP_CUDA(dg.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(dl.alloc(sizeof(double)));
  MLP_CUDA(cudaMemcpy(dX.p, X, sizeof(float) * FRG_MLP_IN * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dy.p, y, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dp.p, params, sizeof(float) * FRG_MLP_NPARAM, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dcw.p, class_w, sizeof(float) * FRG_MLP_OUT, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemset(dg.p, 0, sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(cudaMemset(dl.p, 0, sizeof(double)));
  to_bf16_kernel<<<blocks_for(FRG_MLP_NPARAM, 256), 256>>>((float*)dp.p, (__nv_bfloat16*)dw.p, FRG_MLP_NPARAM);
  grad_kernel<<<blocks_for(n, kThreads), kThreads>>>((float*)dX.p, (int32_t*)dy.p, nullptr, n,
                                                     (__nv_bfloat16*)dw.p, (float*)dcw.p, (float*)dg.p,
                                                     (double*)dl.p);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpy(grad, dg.p, sizeof(float) * FRG_MLP_NPARAM, cudaMemcpyDeviceToHost));
  MLP_CUDA(cudaMemcpy(loss, dl.p, sizeof(double), cudaMemcpyDeviceToHost));
  return FRG_OK;
}

extern "C" frg_status frg_mlp_train(const float* X, const int32_t* y, int64_t n, const float* class_w, int epochs,
                                    int batch, float lr, uint64_t seed, float* params, double* epoch_loss) {
  if (!X || !y || n < 1 || !class_w || epochs < 1 || batch < 1 || !(lr > 0.f) || !params) return FRG_ERR_ARG;
  Dev dX, dy, dp, dw, dcw, dg, dl, dm, dv, didx;
  MLP_CUDA(dX.alloc(sizeof(float) * FRG_MLP_IN * n));
  MLP_CUDA(dy.alloc(sizeof(int32_t) * n));
  MLP_CUDA(dp.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(dw.alloc(sizeof(__nv_bfloat16) * FRG_MLP_NPARAM));
  MLP_CUDA(dcw.alloc(sizeof(float) * FRG_MLP_OUT));
  MLP_CUDA(dg.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(dl.alloc(sizeof(double)));
  MLP_CUDA(dm.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(dv.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(didx.alloc(sizeof(int64_t) * n));
  MLP_CUDA(cudaMemcpy(dX.p, X, sizeof(float) * FRG_MLP_IN * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dy.p, y, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dcw.p, class_w, sizeof(float) * FRG_MLP_OUT, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemset(dm.p, 0, sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(cudaMemset(dv.p, 0, sizeof(float) * FRG_MLP_NPARAM));
  std::mt19937_64 rng(seed);
  // initial weights: the caller's when they are finite and not all zero, else He-normal
  bool given = false;
  for (int i = 0; i < FRG_MLP_NPARAM; ++i) given |= params[i] != 0.f;
  std::vector<float> p0(params, params + FRG_MLP_NPARAM);
  if (!given) {
    std::normal_distribution<float> nd(0.f, 1.f);
    for (int i = 0; i < FRG_MLP_H * FRG_MLP_IN; ++i) p0[FRG_MLP_W1 + i] = nd(rng) * std::sqrt(2.f / FRG_MLP_IN);
    for (int i = 0; i < FRG_MLP_H * FRG_MLP_H; ++i) p0[FRG_MLP_W2 + i] = nd(rng) * std::sqrt(2.f / FRG_MLP_H);
    for (int i = 0; i < FRG_MLP_OUT * FRG_MLP_H; ++i) p0[FRG_MLP_W3 + i] = nd(rng) * std::sqrt(1.f / FRG_MLP_H);
  }
  MLP_CUDA(cudaMemcpy(dp.p, p0.data(), sizeof(float) * FRG_MLP_NPARAM, cudaMemcpyHostToDevice));
  std::vector<int64_t> idx(n);
  for (int64_t i = 0; i < n; ++i) idx[i] = i;
  int t = 0;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(idx.begin(), idx.end(), rng);
    MLP_CUDA(cudaMemcpy(didx.p, idx.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemset(dl.p, 0, sizeof(double)));
    int64_t nb = 0;
    for (int64_t off = 0; off < n; off += batch, ++nb) {
      const int64_t B = std::min<int64_t>(batch, n - off);
      to_bf16_kernel<<<blocks_for(FRG_MLP_NPARAM, 256), 256>>>((float*)dp.p, (__nv_bfloat16*)dw.p, FRG_MLP_NPARAM);
      MLP_CUDA(cudaMemsetAsync(dg.p, 0, sizeof(float) * FRG_MLP_NPARAM));
      grad_kernel<<<blocks_for(B, kThreads), kThreads>>>((float*)dX.p, (int32_t*)dy.p, (int64_t*)didx.p + off, B,
                                                         (__nv_bfloat16*)dw.p, (float*)dcw.p, (float*)dg.p,
                                                         (double*)dl.p);
      ++t;
      adam_kernel<<<blocks_for(FRG_MLP_NPARAM, 256), 256>>>((float*)dp.p, (float*)dg.p, (float*)dm.p, (float*)dv.p,
                                                            FRG_MLP_NPARAM, lr, b1, b2, 1e-8f,
                                                            1.f - std::pow(b1, (float)t), 1.f - std::pow(b2, (float)t));
    }
    MLP_CUDA(cudaGetLastError());
    double l = 0.0;
    MLP_CUDA(cudaMemcpy(&l, dl.p, sizeof(double), cudaMemcpyDeviceToHost));
    if (epoch_loss) epoch_loss[ep] = l / (double)nb;
  }
  MLP_CUDA(cudaMemcpy(params, dp.p, sizeof(float) * FRG_MLP_NPARAM, cudaMemcpyDeviceToHost));
  return FRG_OK;
}

extern "C" frg_status frg_mlp_predict(const float* X, int64_t n, const float* params, float* probs) {
  if (!X || n < 1 || !params || !probs) return FRG_ERR_ARG;
  Dev dX, dp, dw, dpr;
  MLP_CUDA(dX.alloc(sizeof(float) * FRG_MLP_IN * n));
  MLP_CUDA(dp.alloc(sizeof(float) * FRG_MLP_NPARAM));
  MLP_CUDA(dw.alloc(sizeof(__nv_bfloat16) * FRG_MLP_NPARAM));
  MLP_CUDA(dpr.alloc(sizeof(float) * FRG_MLP_OUT * n));
  MLP_CUDA(cudaMemcpy(dX.p, X, sizeof(float) * FRG_MLP_IN * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dp.p, params, sizeof(float) * FRG_MLP_NPARAM, cudaMemcpyHostToDevice));
  to_bf16_kernel<<<blocks_for(FRG_MLP_NPARAM, 256), 256>>>((float*)dp.p, (__nv_bfloat16*)dw.p, FRG_MLP_NPARAM);
  predict_kernel<<<blocks_for(n, 128), 128>>>((float*)dX.p, n, (__nv_bfloat16*)dw.p, (float*)dpr.p);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpy(probs, dpr.p, sizeof(float) * FRG_MLP_OUT * n, cudaMemcpyDeviceToHost));
  return FRG_OK;
}
