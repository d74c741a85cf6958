// Internal declarations of the learned-warm-start MLP (mlp.cu, mlp_train.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mfgb {

constexpr int MLP_IN = 16;   // 10 whitened samples / |y|, log SNR, pederr, 4 zero pads
constexpr int MLP_H = 128;
constexpr int MLP_OUT = 32;  // 10 logits, 10 amplitude outputs, 12 zero pads

enum GemmEpilogue { EPI_BIAS_RELU = 0, EPI_BIAS = 1, EPI_STORE = 2, EPI_ATOMIC = 3 };

// C[M x N] = op(A)[M x K] * op(B)[N x K]^T; element (i,k) of op(A) is
// A[i*a_si + k*a_sk], element (j,k) of op(B) is B[j*b_sj + k*b_sk].
struct GemmArgs {
  const __nv_bfloat16* A;
  int64_t a_si, a_sk;
  const __nv_bfloat16* B;
  int64_t b_sj, b_sk;
  int M, N, K;
  int k_split;  // K range of one grid.z slice
  float* C;
  int ldc;
  const float* bias;
  __nv_bfloat16* H;  // EPI_BIAS_RELU: bf16 ReLU output
  int ldh;
  unsigned* err;     // error word: MLP_ERR_TRAIN_TIMEOUT when a tensor-core wait gives up
  int test_stall;    // wait first on an mbarrier nothing arrives on (timeout test)
};

struct MlpFeatArgs {
  int64_t n;
  int sample_stride;
  const double* samples;
  const double* pederr;
  const uint8_t* ctype;
  int set;  // condition set served by the MLP
  int N;
  float W32[55];
  __nv_bfloat16* X;  // [n][MLP_IN]
  float* scale;      // [n] |y|
};

struct MlpInferArgs {
  int64_t n;
  int sample_stride;
  const double* samples;
  const double* pederr;
  const uint8_t* ctype;
  int set;
  float W32[55];
  float inv_gnorm[10];
  const __nv_bfloat16* W1;  // [MLP_H][MLP_IN]
  const __nv_bfloat16* W2;  // [MLP_H][MLP_H]
  const __nv_bfloat16* W3;  // [MLP_OUT][MLP_H]
  const float* b1;
  const float* b2;
  const float* b3;
  uint16_t* warm_mask;  // [n]
  float* warm_amp;      // [n][warm_stride]
  int warm_stride;
  float* logits;        // optional [n][MLP_OUT] raw outputs
  unsigned* err;        // device error word (MLP_ERR_* bits), or null
  int test_stall;       // wait first on an mbarrier nothing arrives on (timeout test)
};

// Bits of the inference error word.
constexpr unsigned MLP_ERR_TIMEOUT = 1u;        // a bounded wait of the inference on the tensor cores gave up
constexpr unsigned MLP_ERR_TRAIN_TIMEOUT = 2u;  // ... of a training GEMM

__global__ void mlp_features_kernel(const MlpFeatArgs a);
__global__ void mlp_targets_kernel(int64_t n, const double* amp, int amp_stride, const float* scale,
                                   const float* gnorm, float* T);
__global__ void mlp_loss_kernel(int B, const float* O, const float* T, float amp_weight, __nv_bfloat16* dO,
                                float* loss_sum);
__global__ void relu_backward_kernel(int64_t count, const float* dH, const float* Z, __nv_bfloat16* dZ);
__global__ void bias_grad_kernel(int B, int C, const __nv_bfloat16* dZ, float* db);
__global__ void adam_kernel(int count, float* w, const float* g, float* m, float* v, float lr, float b1, float b2,
                            float eps, float c1, float c2);
__global__ void pack_weights_kernel(const float* w, __nv_bfloat16* wh, __nv_bfloat16* wt, int out, int in);
__global__ void mlp_infer_tc_kernel(const MlpInferArgs a);

cudaError_t launch_gemm(int epi, bool akc, bool bkc, const GemmArgs& p, int splits, cudaStream_t s);
cudaError_t launch_mlp_infer(const MlpInferArgs& a, int sms, cudaStream_t s);
size_t infer_tc_smem_bytes();

}  // namespace mfgb
