// Learned warm start: a small MLP that predicts, from the whitened samples and
// the noise scale, the passive set and the amplitudes of a channel's fit.
//
// Network: 16 inputs (10 normalised whitened samples, log SNR, pederr, zero
// padding) -> 128 -> ReLU -> 128 -> ReLU -> 32 outputs (10 passive-set logits,
// 10 amplitude outputs, padding). BF16 weights and activations on the tensor
// cores, FP32 accumulate; FP32 master weights, Adam. Training and inference
// (mlp_tc.cu) both run their GEMMs on tcgen05 with FP32 accumulators in TMEM.
//
// Kernels:
//   mlp_features_kernel   channel -> feature row (bf16) + per-channel scale
//   gemm_tc_kernel<EPI,..> C = A * B^T for every training GEMM (forward layers,
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
#include "tc_common.cuh"

namespace mfgb {
namespace {

typedef __nv_bfloat16 bf16;

using namespace tc;

// Training GEMM on the 5th-generation tensor cores: one CTA of 128 threads
// computes a 128 x 32 tile of C (rows m0.., columns j0..; one TMEM
// accumulator of 128 lanes x 32 columns). Per round the threads stage up to
// 64 of its K into shared memory in the no-swizzle K-major layout (element
// (i, k) of op(X) is X[i*si + k*sk]; KC picks the coalescing direction: k
// contiguous -- then 16-byte loads, one core-matrix row each -- or i
// contiguous for the transposed operands of the weight gradients;
// out-of-range elements are zero), one thread issues the round's
// tcgen05.mma (M = 128, N = 16 or 32, K = 16 per instruction) and commits it
// to the CTA's mbarrier, and all wait for it before the next staging. The
// epilogue reads the accumulator back with tcgen05.ld: warp w holds rows
// 32 w .. 32 w + 31. A wait that gives up (0.2 s) sets MLP_ERR_TRAIN_TIMEOUT
// in the error word, waits once more (bounded) for the MMAs in flight, skips
// the epilogue and frees the TMEM (test_stall makes the first wait give up
// after 1 ms on an mbarrier nothing arrives on).
constexpr int TM = 128;  // rows per CTA = MMA M = TMEM lanes
constexpr int TN = 32;   // columns per CTA
constexpr int TKC = 64;  // K staged per round
constexpr uint32_t kGemmTmemCols = 32;
constexpr uint64_t kGemmWaitNs = 200000000ull;

constexpr uint64_t kGemmTestWaitNs = 1000000ull;  // the timeout test's wait: 1 ms

struct GemmSmem {
  bf16 A[TM * TKC];  // 16 KB
  bf16 B[TN * TKC];  // 4 KB
  unsigned long long bar;
  unsigned long long never;  // nothing arrives on it (the timeout test's wait)
  uint32_t tmem;
};
// at most 10 CTAs of this size fit an SM's shared memory: 10 x 32 TMEM
// columns, within the SM's 512, so tcgen05.alloc never waits
constexpr size_t kGemmSmem = sizeof(GemmSmem);
static_assert(233472 / (kGemmSmem + 1024) * kGemmTmemCols <= 512, "TMEM per SM");

extern __shared__ __align__(128) unsigned char gemm_smem_raw[];

template <bool KC>
__device__ __forceinline__ void stage_tile(bf16* S, const bf16* X, int64_t si, int64_t sk, int i0, int k0, int I,
                                           int kend, int rows, int kc) {
  unsigned char* base = reinterpret_cast<unsigned char*>(S);
  if (KC && sk == 1 && si % 8 == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0) {
    // 8 consecutive k of a row = one 16-byte core-matrix row
    const int groups = kc / 8;
    for (int e = threadIdx.x; e < rows * groups; e += blockDim.x) {
      const int i = e / groups, g = e % groups;
      const int gi = i0 + i, gk = k0 + 8 * g;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gi < I) {
        const bf16* src = X + int64_t(gi) * si + gk;
        if (gk + 8 <= kend) {
          v = *reinterpret_cast<const uint4*>(src);
        } else {
          bf16 t[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) t[q] = gk + q < kend ? src[q] : __float2bfloat16(0.f);
          v = *reinterpret_cast<const uint4*>(t);
        }
      }
      *reinterpret_cast<uint4*>(base + kmaj(i, 8 * g, kc)) = v;
    }
    return;
  }
  for (int e = threadIdx.x; e < rows * kc; e += blockDim.x) {
    int i, k;
    if (KC) {
      i = e / kc;
      k = e % kc;
    } else {
      k = e / rows;
      i = e % rows;
    }
    const int gi = i0 + i, gk = k0 + k;
    bf16 v = __float2bfloat16(0.f);
    if (gi < I && gk < kend) v = X[int64_t(gi) * si + int64_t(gk) * sk];
    *reinterpret_cast<bf16*>(base + kmaj(i, k, kc)) = v;
  }
}

template <int EPI, bool AKC, bool BKC>
__global__ void __launch_bounds__(128) gemm_tc_kernel(const GemmArgs p) {
  GemmSmem& S = *reinterpret_cast<GemmSmem*>(gemm_smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TM, j0 = blockIdx.y * TN;
  const int ncols = min(TN, p.N - j0);
  const int ntile = (ncols + 15) & ~15;  // MMA N: 16 or 32
  const int kbeg = blockIdx.z * p.k_split;
  const int kend = min(p.K, kbeg + p.k_split);
  const uint32_t bar = smem_u32(&S.bar), never = smem_u32(&S.never);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(never) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                 "r"(kGemmTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  const uint32_t id = idesc_bf16(TM, ntile);
  constexpr uint64_t kStep = 256 >> 4;  // descriptor advance of one K = 16 step
  const bf16* Bj = p.B + int64_t(j0) * p.b_sj;
  uint32_t phase = 0;
  bool ok = true, any = false;
  for (int k0 = kbeg; k0 < kend; k0 += TKC) {
    const int kc = min(TKC, (kend - k0 + 15) & ~15);  // this round's K: 16, 32, 48 or 64
    stage_tile<AKC>(S.A, p.A, p.a_si, p.a_sk, m0, k0, p.M, kend, TM, kc);
    stage_tile<BKC>(S.B, Bj, p.b_sj, p.b_sk, 0, k0, ncols, kend, ntile, kc);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint64_t dA = sdesc(smem_u32(S.A), 128, uint32_t(kc) * 16);
      const uint64_t dB = sdesc(smem_u32(S.B), 128, uint32_t(kc) * 16);
      for (int kk = 0; kk < kc / 16; ++kk)
        mma_bf16_tc(tmem, dA + kk * kStep, dB + kk * kStep, id, (any || kk > 0) ? 1u : 0u);
      mma_commit(bar);
    }
    any = true;
    ok = __syncthreads_and(p.test_stall ? mbar_wait(never, 0u, kGemmTestWaitNs) : mbar_wait(bar, phase, kGemmWaitNs));
    if (!ok) break;
    phase ^= 1u;
    tc_fence_after();
  }
  if (!ok) {
    if (tid == 0 && p.err) atomicOr(p.err, MLP_ERR_TRAIN_TIMEOUT);
    mbar_wait(bar, phase, kGemmWaitNs);
  } else if (any) {
    const int row = m0 + warp * 32 + lane;
    const bool live = row < p.M;
    for (int c0 = 0; c0 < ntile; c0 += 16) {
      uint32_t r[16];
      __syncwarp();  // the TMEM load is warp-wide
      tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), r);
      if (live) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (c0 + j >= ncols) break;
          const int c = j0 + c0 + j;
          const float v = __uint_as_float(r[j]);
          if (EPI == EPI_BIAS_RELU) {
            const float z = v + p.bias[c];
            p.C[int64_t(row) * p.ldc + c] = z;
            p.H[int64_t(row) * p.ldh + c] = __float2bfloat16(relu(z));
          } else if (EPI == EPI_BIAS) {
            p.C[int64_t(row) * p.ldc + c] = v + p.bias[c];
          } else if (EPI == EPI_STORE) {
            p.C[int64_t(row) * p.ldc + c] = v;
          } else {  // EPI_ATOMIC: split-K accumulation of a weight gradient
            atomicAdd(&p.C[int64_t(row) * p.ldc + c], v);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kGemmTmemCols) : "memory");
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
  if (p.N < 1 || p.M < 1 || p.K < 1 || p.k_split < 1 || splits < 1) return cudaErrorInvalidValue;
  const dim3 grid(unsigned((p.M + TM - 1) / TM), unsigned((p.N + TN - 1) / TN), unsigned(splits));
#define MF_GEMM_CASE(E, A, B)                                                \
  if (epi == E && akc == A && bkc == B) {                                    \
    gemm_tc_kernel<E, A, B><<<grid, 128, kGemmSmem, s>>>(p);                 \
    return cudaGetLastError();                                               \
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
