// Learned warm start: a small MLP that predicts, from the whitened samples and
// the noise scale, the passive set and the amplitudes of a channel's fit.
//
// Network: 16 inputs (10 normalised whitened samples, log SNR, pederr, zero
// padding) -> 128 -> ReLU -> 128 -> ReLU -> 32 outputs (10 passive-set logits,
// 10 amplitude outputs, padding). BF16 weights and activations on the tensor
// cores, FP32 accumulate; FP32 master weights, Adam. Training runs its GEMMs
// as mma.sync m16n8k16 tiles; inference runs on tcgen05 (mlp_tc.cu).
//
// Kernels:
//   mlp_features_kernel   channel -> feature row (bf16) + per-channel scale
//   gemm_kernel<EPI,..>   C = A * B^T for every training GEMM (forward layers,
//                         input gradients, split-K weight gradients)
//   loss_kernel           BCE on the logits + MSE on softplus(amplitude outputs)
//   relu_backward_kernel, bias_grad_kernel, adam_kernel, pack_weights_kernel
//   launch_mlp_infer      the inference kernel of mlp_tc.cu (the path inside
//                         a timed fit)
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "mf_internal.h"
#include "mlp.h"
#include "mlp_common.cuh"

namespace mfgb {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

// Warp-level 32x32 tile product over one BK slice held in shared memory
// (row-major [rows][BK+PAD], k contiguous), accumulating into acc[2][4][4].
__device__ __forceinline__ void warp_tile_mma(const bf16 (*As)[BK + PAD], const bf16 (*Bs)[BK + PAD], int wm, int wn,
                                              float (&acc)[2][4][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kk = 0; kk < BK; kk += 16) {
    uint32_t a[2][4], b[4][2];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
      const int r = wm + mi * 16 + g;
      a[mi][0] = ld32(&As[r][kk + 2 * t]);
      a[mi][1] = ld32(&As[r + 8][kk + 2 * t]);
      a[mi][2] = ld32(&As[r][kk + 8 + 2 * t]);
      a[mi][3] = ld32(&As[r + 8][kk + 8 + 2 * t]);
    }
#pragma unroll
    for (int ni = 0; ni < 4; ++ni) {
      const int c = wn + ni * 8 + g;
      b[ni][0] = ld32(&Bs[c][kk + 2 * t]);
      b[ni][1] = ld32(&Bs[c][kk + 8 + 2 * t]);
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], a[mi], b[ni]);
  }
}

// Loads a BM x BK (or BN x BK) tile of op(X) into shared memory. Element
// (i, k) of op(X) is X[i*si + k*sk]; KC selects the coalescing direction
// (k contiguous or i contiguous). Out-of-range elements are zero.
template <bool KC, int ROWS>
__device__ __forceinline__ void load_tile(bf16 (*S)[BK + PAD], const bf16* X, int64_t si, int64_t sk, int i0, int k0,
                                          int I, int Kend) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int e = tid; e < ROWS * BK; e += 128) {
    int i, k;
    if (KC) {
      i = e / BK;
      k = e % BK;
    } else {
      k = e / ROWS;
      i = e % ROWS;
    }
    const int gi = i0 + i, gk = k0 + k;
    bf16 v = __float2bfloat16(0.f);
    if (gi < I && gk < Kend) v = X[gi * si + gk * sk];
    S[i][k] = v;
  }
}

template <int EPI, bool AKC, bool BKC>
__global__ void __launch_bounds__(128) gemm_kernel(const GemmArgs p) {
  __shared__ __align__(16) bf16 As[BM][BK + PAD];
  __shared__ __align__(16) bf16 Bs[BN][BK + PAD];
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kbeg = blockIdx.z * p.k_split;
  const int kend = min(p.K, kbeg + p.k_split);
  const int warp = threadIdx.x >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4] = {};
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    load_tile<AKC, BM>(As, p.A, p.a_si, p.a_sk, m0, k0, p.M, kend);
    load_tile<BKC, BN>(Bs, p.B, p.b_sj, p.b_sk, n0, k0, p.N, kend);
    __syncthreads();
    warp_tile_mma(As, Bs, wm, wn, acc);
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int r = m0 + wm + mi * 16 + g + (h >= 2 ? 8 : 0);
        const int c = n0 + wn + ni * 8 + 2 * t + (h & 1);
        if (r >= p.M || c >= p.N) continue;
        const float v = acc[mi][ni][h];
        if (EPI == EPI_BIAS_RELU) {
          const float z = v + p.bias[c];
          p.C[int64_t(r) * p.ldc + c] = z;
          p.H[int64_t(r) * p.ldh + c] = __float2bfloat16(relu(z));
        } else if (EPI == EPI_BIAS) {
          p.C[int64_t(r) * p.ldc + c] = v + p.bias[c];
        } else if (EPI == EPI_STORE) {
          p.C[int64_t(r) * p.ldc + c] = v;
        } else {  // EPI_ATOMIC: split-K accumulation of a weight gradient
          atomicAdd(&p.C[int64_t(r) * p.ldc + c], v);
        }
      }
}

}  // namespace

// --------------------------------------------------------------------------
// element-wise kernels
// --------------------------------------------------------------------------

// Features of channel i: y = L_R^-1 s (FP64), f = [y/|y|, log(|y|/sigma)/10,
// sigma, 0...]; scale[i] = |y| (the amplitude outputs are in units of
// |y| / |G_k|). Channels of a set without tables (HCAL here) get f = 0.
__global__ void mlp_features_kernel(const MlpFeatArgs a) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= a.n) return;
  float f[MLP_IN];
  for (int j = 0; j < MLP_IN; ++j) f[j] = 0.f;
  float scale = 0.f;
  const int t = a.ctype ? int(a.ctype[i]) : 0;
  if (t == a.set && a.N == 10) mlp_features(a.W32, a.samples + i * a.sample_stride, a.pederr[i], f, &scale);
  bf16* out = a.X + i * MLP_IN;
  for (int j = 0; j < MLP_IN; ++j) out[j] = __float2bfloat16(f[j]);
  if (a.scale) a.scale[i] = scale;
}

// Targets from a converged fit: support bit and t_k = x_k |G_k| / |y|.
__global__ void mlp_targets_kernel(int64_t n, const double* amp, int amp_stride, const float* scale,
                                   const float* gnorm, float* T) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float sc = scale[i];
  for (int k = 0; k < 10; ++k) {
    const double x = amp[i * amp_stride + k];
    T[i * 20 + k] = x > 0. ? 1.f : 0.f;
    T[i * 20 + 10 + k] = sc > 0.f ? float(x * gnorm[k] / sc) : 0.f;
  }
}

// Loss of a batch and its gradient dO (bf16, already divided by the batch).
__global__ void mlp_loss_kernel(int B, const float* O, const float* T, float amp_weight, bf16* dO,
                                float* loss_sum) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  float l = 0.f;
  const float invB = 1.f / float(B);
  for (int k = 0; k < 10; ++k) {
    const float z = O[i * MLP_OUT + k], y = T[i * 20 + k];
    l += fmaxf(z, 0.f) - z * y + log1pf(expf(-fabsf(z)));
    dO[i * MLP_OUT + k] = __float2bfloat16((sigmoidf(z) - y) * invB);
    const float o = O[i * MLP_OUT + 10 + k], tt = T[i * 20 + 10 + k];
    const float sp = softplusf(o), d = sp - tt;
    l += amp_weight * d * d;
    dO[i * MLP_OUT + 10 + k] = __float2bfloat16(2.f * amp_weight * d * sigmoidf(o) * invB);
  }
  for (int k = 20; k < MLP_OUT; ++k) dO[i * MLP_OUT + k] = __float2bfloat16(0.f);
  if (loss_sum) atomicAdd(loss_sum, l * invB);
}

__global__ void relu_backward_kernel(int64_t count, const float* dH, const float* Z, bf16* dZ) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  dZ[i] = __float2bfloat16(dH[i] * relu_grad(Z[i]));
}

// db[c] += sum_b dZ[b][c] over a chunk of rows (float atomics).
__global__ void bias_grad_kernel(int B, int C, const bf16* dZ, float* db) {
  const int c = threadIdx.x;
  if (c >= C) return;
  const int rows = (B + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * rows, r1 = min(B, r0 + rows);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += __bfloat162float(dZ[int64_t(r) * C + c]);
  atomicAdd(&db[c], s);
}

__global__ void adam_kernel(int count, float* w, const float* g, float* m, float* v, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// FP32 master weights -> BF16 copies (row-major [out][in]) and their transposes.
__global__ void pack_weights_kernel(const float* w, bf16* wh, bf16* wt, int out, int in) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= out * in) return;
  const int o = i / in, c = i % in;
  const bf16 v = __float2bfloat16(w[i]);
  wh[i] = v;
  if (wt) wt[c * out + o] = v;
}

// --------------------------------------------------------------------------
// launchers
// --------------------------------------------------------------------------
cudaError_t launch_gemm(int epi, bool akc, bool bkc, const GemmArgs& p, int splits, cudaStream_t s) {
  dim3 grid((p.N + BN - 1) / BN, (p.M + BM - 1) / BM, splits);
#define MF_GEMM_CASE(E, A, B)                                          \
  if (epi == E && akc == A && bkc == B) {                              \
    gemm_kernel<E, A, B><<<grid, 128, 0, s>>>(p);                      \
    return cudaGetLastError();                                         \
  }
  MF_GEMM_CASE(EPI_BIAS_RELU, true, true)
  MF_GEMM_CASE(EPI_BIAS, true, true)
  MF_GEMM_CASE(EPI_STORE, true, true)
  MF_GEMM_CASE(EPI_ATOMIC, false, false)
#undef MF_GEMM_CASE
  return cudaErrorInvalidValue;
}

// The tensor-core inference kernel (mlp_tc.cu): one wave of persistent CTAs
// of 512 threads, two per SM (each holds 256 of the SM's 512 TMEM columns and
// half of its shared memory for its lifetime).
cudaError_t launch_mlp_infer(const MlpInferArgs& a, int sms, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  static bool attr_set = false;
  const size_t smem = infer_tc_smem_bytes();
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int64_t tiles = (a.n + 127) / 128;
  const int64_t cap = 2 * int64_t(sms);
  const int grid = int(tiles < cap ? tiles : cap);
  mlp_infer_tc_kernel<<<grid, 512, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mfgb
