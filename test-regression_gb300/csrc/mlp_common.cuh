// Device helpers shared by the MLP kernels (training and inference).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace mfgb {

// Two floats -> one register holding two BF16 (first in the low half).
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// ReLU hidden units. The network's cost on the GPU is its hidden-layer
// epilogue (256 activations per channel between the tensor-core layers): a
// ReLU is one packed convert-with-clamp per two activations where the tanh
// form of GELU took ~6 FP32 operations and a MUFU tanh each (measured on 10M
// ECAL channels: inference 1.41 ms with GELU, 1.00 ms with ReLU; fit results
// identical, the warm fit 5% faster end to end).
__device__ __forceinline__ float relu(float x) { return fmaxf(x, 0.f); }
__device__ __forceinline__ float relu_grad(float x) { return x > 0.f ? 1.f : 0.f; }
// A column enters the predicted passive set when its logit exceeds -0.5
// (probability 0.38, not 0.5): a column predicted needlessly costs the warm
// FP32 search one drop step, a column missed costs a fix and a second judge
// (measured on 10M ECAL channels: 8.48 ms per fit at -0.5, 8.90 ms at 0,
// 8.55 ms at -1, 9.34 ms at -2).
constexpr float kMaskLogit = -0.5f;

__device__ __forceinline__ float softplusf(float x) { return x > 20.f ? x : log1pf(expf(x)); }
__device__ __forceinline__ float sigmoidf(float x) { return 1.f / (1.f + expf(-x)); }

// MLP input of a channel, in FP32 (the network reads BF16): y = L_R^-1 s from
// the FP32 inverse factor (packed rows, N = 10), f[0..9] = y / |y|,
// f[10] = log(|y| / pederr) / 10, f[11] = pederr, f[12..15] = 0; *scale = |y|
// (the amplitude outputs are in units of |y| / |G_k|). The one definition used
// by training and inference.
__device__ __forceinline__ void mlp_features(const float* W32, const double* s, double pederr, float* f,
                                             float* scale) {
  float y[10], n2 = 0.f;
  int w = 0;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c <= r; ++c) acc = fmaf(W32[w + c], float(s[c]), acc);
    w += r + 1;
    y[r] = acc;
    n2 = fmaf(acc, acc, n2);
  }
  const float nrm = sqrtf(n2);
  const float inv = nrm > 0.f ? 1.f / nrm : 0.f;
  const float sig = float(pederr);
#pragma unroll
  for (int r = 0; r < 10; ++r) f[r] = y[r] * inv;
  f[10] = logf(fmaxf(nrm / sig, 1e-30f)) * 0.1f;
  f[11] = sig;
#pragma unroll
  for (int r = 12; r < 16; ++r) f[r] = 0.f;
  *scale = nrm;
}

}  // namespace mfgb
