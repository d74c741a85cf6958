// Warm-start MLP inference on the 5th-generation tensor cores (tcgen05).
//
// One CTA of 512 threads (four warpgroups; two CTAs per SM) fits tiles of
// 128 channels, persistent over the batch, two tiles at a time (slots 0 and 1, each with
// its own 128 TMEM columns, shared-memory A operand and mbarrier). Per tile
// the three layers are three rounds of
//   one thread issues tcgen05.mma (BF16 operands from shared memory, FP32
//   accumulators in tensor memory), commits them to the slot's mbarrier;
//   warp w reads TMEM lanes 32 (w % 4) .. +31 (= 32 channels; a warp may only
//   read its quarter of the lanes) and the 32 columns of warpgroup w / 4, adds
//   the bias, applies the ReLU and writes the BF16 activations back to shared
//   memory as the A operand of the next layer,
// and the slots alternate: while the tensor cores run one slot's layer, the
// warps run the other slot's epilogue. Warpgroup 0 also computes the
// features and decodes the outputs (one channel per thread). The network's weights are staged once
// per CTA. Nothing of the MMA passes through registers: the CUDA cores run
// only the features, the bias+ReLU epilogues and the decode of the outputs.
//
// Shared-memory operands in the no-swizzle K-major layout of tc_common.cuh.
//
// Every wait on the MMA completion is bounded (globaltimer). A tile whose
// wait gives up sets bit MLP_ERR_TIMEOUT of the error word, waits (bounded)
// for the MMAs in flight, and the CTA predicts the empty set for the rest of
// its tiles (a cold start: the fit's result does not depend on the
// prediction) before it frees its tensor memory and returns.
#include <cuda_bf16.h>

#include "mlp.h"
#include "mlp_common.cuh"
#include "tc_common.cuh"

namespace mfgb {
namespace {

using namespace tc;

typedef __nv_bfloat16 bf16;

constexpr int TILE = 128;             // channels per tile = MMA M = TMEM lanes
constexpr int kThreads = 512;         // four warpgroups, 32 columns of every layer each
constexpr uint32_t kTmemCols = 256;   // per slot: D of every layer (layer 3 uses its first 32 columns)
constexpr uint64_t kWaitNs = 200000000ull;  // 0.2 s: an MMA round takes ~1 us
constexpr uint64_t kTestWaitNs = 1000000ull;  // the timeout test's wait: 1 ms

extern __shared__ __align__(128) unsigned char tc_smem_raw[];

struct TcSmem {
  bf16 W2[MLP_H * MLP_H];    // B of layer 2: N = 128, K = 128 (32 KB)
  bf16 H[2][TILE * MLP_H];   // A per slot: the features (K = 16), then H1, then H2 (K = 128)
  bf16 W3[MLP_OUT * MLP_H];  // B of layer 3: N = 32, K = 128
  bf16 W1[MLP_H * MLP_IN];   // B of layer 1: N = 128, K = 16
  float b1[MLP_H], b2[MLP_H], b3[MLP_OUT];
  float scale[2][2][TILE];   // |y| of each slot's channels, features -> decode (by pair parity)
  unsigned long long bar[2]; // MMA completion per slot
  unsigned long long never;  // nothing arrives on it (the timeout test's wait)
  uint32_t tmem;             // TMEM base written by tcgen05.alloc
};

// Starts moving the line holding p into L2 (no register is written).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// max(lo, 0) and max(hi, 0) rounded to BF16 and packed, lo in the low half:
// one instruction (the PTX convert packs its first operand in the high half).
__device__ __forceinline__ uint32_t pack_relu_bf16(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// 32 columns (this warpgroup's) of a layer's output for this thread's channel
// (TMEM lane = row) -> bias + ReLU -> BF16 into the next layer's A operand
// (K = 128): k groups 4 cg .. 4 cg + 3 of the row, 16 columns at a time.
__device__ __forceinline__ void relu_epilogue(uint32_t tm, const float* bias, uint32_t hrow) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    uint32_t r[16];
    tmem_ld16(tm + 16u * half, r);
    uint32_t p[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 bb = *reinterpret_cast<const float4*>(bias + 16 * half + 4 * q);
      p[2 * q] = pack_relu_bf16(__uint_as_float(r[4 * q]) + bb.x, __uint_as_float(r[4 * q + 1]) + bb.y);
      p[2 * q + 1] = pack_relu_bf16(__uint_as_float(r[4 * q + 2]) + bb.z, __uint_as_float(r[4 * q + 3]) + bb.w);
    }
    st_shared_v4(hrow + (2 * half) * 128, p[0], p[1], p[2], p[3]);
    st_shared_v4(hrow + (2 * half + 1) * 128, p[4], p[5], p[6], p[7]);
  }
}

// softplus with the hardware exp2/log2 (relative error ~2^-21): the
// amplitudes only seed the FP32 search.
__device__ __forceinline__ float softplus_fast(float x) {
  return fmaxf(x, 0.f) + __logf(1.f + __expf(-fabsf(x)));
}

}  // namespace

__global__ void __launch_bounds__(kThreads, 2) mlp_infer_tc_kernel(const MlpInferArgs a) {
  TcSmem& S = *reinterpret_cast<TcSmem*>(tc_smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (TILE - 1), cg = tid >> 7;  // channel of the tile, warpgroup (column block)
  const uint32_t lane_off = uint32_t((warp & 3) * 32) << 16;  // this warp's TMEM lanes
  // weights into the operand layout (16-byte pieces: 8 consecutive k of a row)
  for (int e = tid; e < MLP_H * (MLP_H / 8); e += kThreads) {
    const int n = e / (MLP_H / 8), g = e % (MLP_H / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(a.W2 + n * MLP_H + 8 * g);
    *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.W2) + kmaj(n, 8 * g, MLP_H)) = v;
  }
  for (int e = tid; e < MLP_OUT * (MLP_H / 8); e += kThreads) {
    const int n = e / (MLP_H / 8), g = e % (MLP_H / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(a.W3 + n * MLP_H + 8 * g);
    *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.W3) + kmaj(n, 8 * g, MLP_H)) = v;
  }
  for (int e = tid; e < MLP_H * (MLP_IN / 8); e += kThreads) {
    const int n = e / (MLP_IN / 8), g = e % (MLP_IN / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(a.W1 + n * MLP_IN + 8 * g);
    *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.W1) + kmaj(n, 8 * g, MLP_IN)) = v;
  }
  for (int e = tid; e < MLP_H; e += kThreads) {
    S.b1[e] = a.b1[e];
    S.b2[e] = a.b2[e];
  }
  if (tid < MLP_OUT) S.b3[tid] = a.b3[tid];
  const uint32_t bar0 = smem_u32(&S.bar[0]), bar1 = smem_u32(&S.bar[1]), never = smem_u32(&S.never);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(never) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  const uint64_t dW1 = sdesc(smem_u32(S.W1), 128, MLP_IN * 16);
  const uint64_t dW2 = sdesc(smem_u32(S.W2), 128, MLP_H * 16), dW3 = sdesc(smem_u32(S.W3), 128, MLP_H * 16);
  constexpr uint64_t kStep = 256 >> 4;  // descriptor advance of one K = 16 step
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};  // a commit not yet waited for
  bool dead = false;                 // a wait gave up: predict the empty set from here on

  auto slot_h = [&](int s) { return smem_u32(S.H[s]); };
  auto slot_bar = [&](int s) { return s ? bar1 : bar0; };
  auto slot_tm = [&](int s) { return tmem + 128u * uint32_t(s); };
  // the threads' shared-memory writes and TMEM reads, before the next MMA
  auto stage_sync = [&]() {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  };
  // layer `layer` of slot s on the tensor cores (thread 0), committed to its barrier
  auto issue = [&](int s, int layer) {
    if (tid == 0) {
      const uint32_t d = slot_tm(s), h = slot_h(s);
      if (layer == 1) {
        mma_bf16_tc(d, sdesc(h, 128, MLP_IN * 16), dW1, idesc_bf16(TILE, MLP_H), 0u);
      } else {
        const uint64_t dA = sdesc(h, 128, MLP_H * 16), dB = layer == 2 ? dW2 : dW3;
        const uint32_t id = idesc_bf16(TILE, layer == 2 ? MLP_H : MLP_OUT);
#pragma unroll
        for (int kk = 0; kk < MLP_H / 16; ++kk) mma_bf16_tc(d, dA + kk * kStep, dB + kk * kStep, id, kk > 0);
      }
      mma_commit(slot_bar(s));
    }
    pending[s] = true;
  };
  // everyone waits for slot s's last commit; false (for every thread) if it gave up
  auto wait = [&](int s) -> bool {
    const bool ok = a.test_stall ? mbar_wait(never, 0u, kTestWaitNs) : mbar_wait(slot_bar(s), phase[s], kWaitNs);
    const bool all_ok = __syncthreads_and(ok);
    if (all_ok) {
      phase[s] ^= 1u;
      pending[s] = false;
      tc_fence_after();
    }
    return all_ok;
  };
  // features of channel i into slot s's A operand (K = 16); *scale = |y|
  auto features = [&](int s, int64_t i, bool mine, float& scale) {
    float f[MLP_IN];
#pragma unroll
    for (int j = 0; j < MLP_IN; ++j) f[j] = 0.f;
    scale = 0.f;
    if (mine) mlp_features(a.W32, a.samples + i * a.sample_stride, a.pederr[i], f, &scale);
    const uint32_t hr = slot_h(s) + kmaj(row, 0, MLP_IN);
    st_shared_v4(hr, pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
    st_shared_v4(hr + 128, pack_bf16(f[8], f[9]), pack_bf16(f[10], f[11]), pack_bf16(f[12], f[13]),
                 pack_bf16(f[14], f[15]));
  };
  auto epilogue = [&](int s, const float* bias) {
    relu_epilogue(slot_tm(s) + lane_off + 32u * cg, bias + 32 * cg, slot_h(s) + kmaj(row, 32 * cg, MLP_H));
  };
  // the outputs of channel i from columns 0..31 of slot s's layer 3
  auto decode = [&](int s, int64_t i, bool mine, float scale) {
    uint32_t r[32], r0[16], r1[16];
    tmem_ld16(slot_tm(s) + lane_off, r0);
    tmem_ld16(slot_tm(s) + lane_off + 16u, r1);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      r[k] = r0[k];
      r[16 + k] = r1[k];
    }
    if (i < a.n) {
      uint16_t m = 0;
      float* wa = a.warm_amp + i * a.warm_stride;
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        const float logit = __uint_as_float(r[k]) + S.b3[k];
        if (logit > kMaskLogit && scale > 0.f) m |= uint16_t(1u << k);
        wa[k] = softplus_fast(__uint_as_float(r[10 + k]) + S.b3[10 + k]) * scale * a.inv_gnorm[k];
      }
      a.warm_mask[i] = mine ? m : uint16_t(0);
      if (a.logits) {
#pragma unroll
        for (int k = 0; k < MLP_OUT; ++k) a.logits[i * MLP_OUT + k] = __uint_as_float(r[k]) + S.b3[k];
      }
    }
  };
  // slot s of pair t0 holds tile t0 + s * gridDim.x; this thread's channel of it
  auto chan = [&](int64_t t0, int s) { return (t0 + s * int64_t(gridDim.x)) * TILE + row; };
  auto owns = [&](int64_t i) { return i < a.n && (a.ctype ? int(a.ctype[i]) : 0) == a.set; };

  // Roles: warpgroups 2 and 3 compute the features of slots 0 and 1 of the
  // next pair while warpgroups 0 and 1 decode slots 0 and 1 of the current
  // one; every warpgroup runs a quarter of each epilogue. The scale |y| of a
  // channel goes from its features thread to its decode thread through
  // shared memory.
  const int64_t tiles = (a.n + TILE - 1) / TILE;
  const int64_t stride = 2 * int64_t(gridDim.x);
  int64_t t0 = blockIdx.x;
  int par = 0;  // scale buffer of the current pair
  if (t0 < tiles && cg >= 2) {
    const int s = cg - 2;
    const int64_t i = chan(t0, s);
    float sc;
    features(s, i, owns(i), sc);
    S.scale[0][s][row] = sc;
  }
  for (; t0 < tiles; t0 += stride) {
    stage_sync();
    issue(0, 1);
    issue(1, 1);
    if (!wait(0)) { dead = true; break; }
    // the samples of the channels whose features this thread computes at the
    // end of this pair start towards L2 now, four stages ahead of their use
    if (cg >= 2 && t0 + stride < tiles) {
      const int64_t i = chan(t0 + stride, cg - 2);
      if (i < a.n) {
        const double* sp = a.samples + i * a.sample_stride;
        prefetch_l2(sp);
        prefetch_l2(sp + 9);  // the row of 10 samples may cross a line
        prefetch_l2(a.pederr + i);
      }
    }
    epilogue(0, S.b1);
    stage_sync();
    issue(0, 2);
    if (!wait(1)) { dead = true; break; }
    epilogue(1, S.b1);
    stage_sync();
    issue(1, 2);
    if (!wait(0)) { dead = true; break; }
    epilogue(0, S.b2);
    stage_sync();
    issue(0, 3);
    if (!wait(1)) { dead = true; break; }
    epilogue(1, S.b2);
    stage_sync();
    issue(1, 3);
    if (!wait(0)) { dead = true; break; }
    if (!wait(1)) { dead = true; break; }
    // the layer-3 MMAs are done: H is free for the next pair's features while
    // TMEM is read by the decode (the barrier at the top of the loop orders
    // both before the next MMAs)
    const int64_t t1 = t0 + stride;
    if (cg < 2) {
      const int64_t i = chan(t0, cg);
      decode(cg, i, owns(i), S.scale[par][cg][row]);
    } else if (t1 < tiles) {
      const int s = cg - 2;
      const int64_t i = chan(t1, s);
      float sc;
      features(s, i, owns(i), sc);
      S.scale[par ^ 1][s][row] = sc;
    }
    par ^= 1;
    tc_fence_before();
  }
  if (dead) {
    // report, let the MMAs in flight finish (bounded) before TMEM is freed,
    // and predict the empty set (a cold start) for this pair and the rest
    if (tid == 0 && a.err) atomicOr(a.err, MLP_ERR_TIMEOUT);
    for (int s = 0; s < 2; ++s)
      if (pending[s]) mbar_wait(slot_bar(s), phase[s], kWaitNs);
    for (; t0 < tiles; t0 += stride) {
      const int64_t i = chan(t0, cg & 1);
      if (cg < 2 && i < a.n) a.warm_mask[i] = 0;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

size_t infer_tc_smem_bytes() { return sizeof(TcSmem); }

}  // namespace mfgb
