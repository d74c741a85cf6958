// Mixed-precision multifit (FP32 active-set search, FP64 judge), and its
// learned-warm-start variant.
//
// Per channel, with the condition set's tables (tables.cu):
//   1. y = L_R^-1 s in FP64 (packed inverse factor: 55 FMA, no division);
//   2. FNNLS active-set search in FP32 (nnls/src/inplace_fnnls.cu:127-231
//      structure: add the column of largest gradient w = c - H x, solve the
//      passive set, step back and drop columns that go non-positive) where
//      every passive-set solve is x_S = G_S^+ y from the FP32 table;
//   3. the same loop continued in FP64 from the FP32 passive set ("the FP64
//      judge"): one FP64 solve with the FP64 pseudo-inverse, which is exact to
//      FP64 rounding, then the KKT test max w < eps * pederr^2 (the reference's
//      absolute eps on the pederr-scaled gradient); a miss of the FP32 search
//      is repaired here, so the result is always the FP64 KKT point;
//   4. chi2 = ||y - G x||^2 / pederr^2 in FP64.
// The covariance does not depend on the amplitudes (no fullpulsecov), so the
// outer chi2 loop of Minimize (multifit_cpu/src/PulseChiSqSNNLS.cpp:149-166)
// would only repeat a KKT-converged fit and confirm delta chi2 = 0: this form
// runs it once.
#include <cfloat>

#include "mf_internal.h"
#include "mlp.h"
#include "mlp_common.cuh"

namespace mfgb {
namespace {

// Passive-set solves from the operator table (tables.cu): rows of the set's
// columns, p x N packed at offset[m]. The loops are predicated on the mask, so
// every lane issues the same instruction stream; only the addresses differ.
template <int N, int K>
__device__ __forceinline__ void solve32(const DevMixed& T, unsigned m, const float* y32, float* s) {
  const float* P = T.pinv32 + __ldg(T.offset + m);
  int r = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float acc = 0.f;
    if (m & (1u << k)) {
      const float2* row = reinterpret_cast<const float2*>(P + r * N);
#pragma unroll
      for (int q = 0; q < N / 2; ++q) {
        const float2 v = __ldg(row + q);
        acc = fmaf(v.x, y32[2 * q], acc);
        acc = fmaf(v.y, y32[2 * q + 1], acc);
      }
      ++r;
    }
    s[k] = acc;
  }
}

template <int N, int K>
__device__ __forceinline__ void solve64(const DevMixed& T, unsigned m, const double* y, double* s) {
  const double* P = T.pinv64 + __ldg(T.offset + m);
  int r = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double acc = 0.;
    if (m & (1u << k)) {
      const double2* row = reinterpret_cast<const double2*>(P + r * N);
#pragma unroll
      for (int q = 0; q < N / 2; ++q) {
        const double2 v = __ldg(row + q);
        acc = fma(v.x, y[2 * q], acc);
        acc = fma(v.y, y[2 * q + 1], acc);
      }
      ++r;
    }
    s[k] = acc;
  }
}

// x > 0 for a finite double, decided on its bit pattern (integer ops, which
// keeps the compare off the FP64 pipe)
__device__ __forceinline__ bool pos64(double v) {
  const int hi = __double2hiint(v);
  const unsigned lo = unsigned(__double2loint(v));
  return (hi > 0 || (hi == 0 && lo != 0u)) && hi < 0x7ff00000;
}

// FNNLS inner loop (nnls/src/inplace_fnnls.cu:175-230) on a bit mask: solve
// the passive set; if some component is not positive, step from the feasible
// x towards s until the first one hits zero and drop it. Returns the solves.
template <int K, typename F, typename Solve>
__device__ __forceinline__ int inner_loop(unsigned& m, F* x, Solve solve) {
  int solves = 0;
  for (int guard = 0; guard <= K && m; ++guard) {
    F s[K];
    solve(m, s);
    ++solves;
    bool allpos = true;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if ((m & (1u << k)) && !(s[k] > F(0))) allpos = false;
    if (allpos) {
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (m & (1u << k)) x[k] = s[k];
      return solves;
    }
    F alpha = F(3.0e38);
    int ai = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((m & (1u << k)) && !(s[k] > F(0))) {
        const F ratio = x[k] / (x[k] - s[k]);
        if (ai < 0 || ratio < alpha) {
          alpha = ratio;
          ai = k;
        }
      }
    }
    if (!(alpha >= F(0))) alpha = F(0);  // 0/0 from a column that entered at zero
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (m & (1u << k)) x[k] = x[k] + alpha * (s[k] - x[k]);
    x[ai] = F(0);
    m &= ~(1u << ai);
  }
  return solves;
}

// Loads a channel and whitens it with the shared inverse factor: y = L_R^-1 s
// in FP64 (packed rows, 55 FMA for N = 10, no division). Returns true for a
// non-finite or non-positive input.
template <int N>
__device__ __forceinline__ bool whiten(const MixedArgs& a, const DevMixed& T, int64_t ch, double* y, double& sig) {
  const double* in = a.samples + ch * a.sample_stride;
  sig = a.pederr[ch];
  bool bad = !isfinite(sig) || !(sig > 0.);
  double s[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    s[i] = in[i];
    bad = bad || !isfinite(s[i]);
  }
  int w = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double acc = 0.;
#pragma unroll
    for (int j = 0; j <= i; ++j) acc = fma(T.W64[w + j], s[j], acc);
    w += i + 1;
    y[i] = acc;
  }
  return bad;
}

// The fit of one whitened channel (steps 2-4), optionally from a predicted
// passive set warm_m with amplitudes warm_x.
// `lanes` = the lanes of the warp that call this function for the same (N, K);
// they reconverge before the FP64 judge, so its FP64 instructions are issued
// once for all of them rather than once per group of lanes that left the
// FP32 search together.
template <int N, int K>
__device__ void fit_from_y(const MixedArgs& a, const DevMixed& T, int64_t ch, const double* y, double sig, bool bad,
                           bool warm, unsigned warm_m, const float* warm_x, unsigned lanes) {
  // executed FP64 flops (FMA = 2): whitening, FP64 solves, residuals, FP64
  // gradients and chi2 -- the work on the FP64 pipe, the bound of this kernel
  int f64 = N * (N + 1);
  float y32[N];
  float ynorm2 = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    y32[i] = float(y[i]);
    ynorm2 = fmaf(y32[i], y32[i], ynorm2);
  }
  // 2. FP32 active-set search
  float c32[K], cmag[K];  // c = G^T y and sum |G_ik y_i| (its FP32 error scale)
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float acc = 0.f, mag = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) {
        acc = fmaf(T.G32[k * N + i], y32[i], acc);
        mag = fmaf(fabsf(T.G32[k * N + i]), fabsf(y32[i]), mag);
      }
    c32[k] = acc;
    cmag[k] = mag;
  }
  const float ynorm = sqrtf(ynorm2);
  const unsigned full = (1u << K) - 1u;
  unsigned m = 0;
  float x32[K];
#pragma unroll
  for (int k = 0; k < K; ++k) x32[k] = 0.f;
  int adds = 0, solves = 0;
  auto s32 = [&](unsigned mm, float* out) { solve32<N, K>(T, mm, y32, out); };
  if (warm) {
    m = warm_m & full;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (m & (1u << k)) x32[k] = fmaxf(warm_x[k], 1e-30f);
    if (m) solves += inner_loop<K>(m, x32, s32);
  }
  for (int it = 0; it < a.max_iter32; ++it) {
    float wmax = 0.f;
    int imax = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (m & (1u << k)) continue;
      float acc = c32[k];
#pragma unroll
      for (int j = 0; j < K; ++j) acc = fmaf(-T.H32[k * KMAX + j], x32[j], acc);
      // relative stop: w_k against |G_k| |y| at the FP32 resolution
      const float tol = a.tol32 * T.gnorm32[k] * ynorm;
      if (acc > tol && (imax < 0 || acc > wmax)) {
        wmax = acc;
        imax = k;
      }
    }
    if (imax < 0) break;
    m |= 1u << imax;
    ++adds;
    solves += inner_loop<K>(m, x32, s32);
  }
  __syncwarp(lanes);
  // 3. FP64 judge, written so that every lane issues the same FP64 work (on
  //    this GPU an FP64 warp instruction costs the full pipe time whatever
  //    the number of active lanes): the dense FP64 solve on the FP32 passive
  //    set, the dense FP64 residual, and the KKT test screened in FP32 with an
  //    FP64 gradient only when some lane of the warp is within the FP32 error
  //    of the threshold. A failed test continues the loop in FP64.
  double x[K];
  auto s64 = [&](unsigned mm, double* out) {
    solve64<N, K>(T, mm, y, out);
    f64 += 2 * N * K;
  };
  {
    double sv[K];
    s64(m, sv);
    ++solves;
    bool allpos = true;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      x[k] = sv[k];
      if ((m & (1u << k)) && !pos64(sv[k])) allpos = false;
    }
    if (!allpos) {  // rare: step back from the feasible FP32 point in FP64
#pragma unroll
      for (int k = 0; k < K; ++k) x[k] = double(x32[k]);
      solves += inner_loop<K>(m, x, s64);
    }
  }
  const double tol64 = a.eps * sig * sig;
  bool converged = false;
  int adds64 = 0;
  double r[N];
  for (int it = 0;; ++it) {
    // FP64 residual r = y - G x (dense: x_k = 0 outside the passive set)
#pragma unroll
    for (int i = 0; i < N; ++i) r[i] = y[i];
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int i = 0; i < N; ++i) r[i] = fma(-T.G64[k * N + i], x[k], r[i]);
    f64 += 2 * N * K;
    if (it >= a.max_iter64) break;
    float xf[K];
#pragma unroll
    for (int k = 0; k < K; ++k) xf[k] = float(x[k]);
    unsigned flagged = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (m & (1u << k)) continue;
      float acc = c32[k], mag = cmag[k];
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const float hx = T.H32[k * KMAX + j] * xf[j];
        acc -= hx;
        mag += fabsf(hx);
      }
      if (acc >= -4e-6f * mag) flagged |= 1u << k;  // not certainly below the threshold
    }
    if (!__any_sync(__activemask(), flagged != 0u)) {  // warp-uniform when converged
      converged = true;
      break;
    }
    double wmax = 0.;
    int imax = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double w = 0.;
#pragma unroll
      for (int i = 0; i < N; ++i) w = fma(T.G64[k * N + i], r[i], w);
      if ((flagged & (1u << k)) && (imax < 0 || w > wmax)) {
        wmax = w;
        imax = k;
      }
    }
    f64 += 2 * N * K;
    if (imax < 0 || !(wmax >= tol64)) {
      converged = true;
      break;
    }
    m |= 1u << imax;
    ++adds64;
    solves += inner_loop<K>(m, x, s64);
  }
  // 4. chi2 in FP64 from the residual
  double chi2 = 0.;
#pragma unroll
  for (int i = 0; i < N; ++i) chi2 = fma(r[i], r[i], chi2);
  chi2 = chi2 / (sig * sig);
  f64 += 2 * N + 2;
  if (a.flops) a.flops[ch] = double(f64);

  double* out = a.amplitudes + ch * a.amp_stride;
  bool finite = isfinite(chi2);
  uint16_t support = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    out[k] = x[k];
    finite = finite && isfinite(x[k]);
    if (x[k] > 0.) support |= uint16_t(1u << k);
  }
  for (int k = K; k < a.amp_stride && k < KMAX; ++k) out[k] = 0.;
  a.chi2[ch] = chi2;
  if (a.intime) a.intime[ch] = T.intime_col >= 0 ? x[T.intime_col] : 0.;
  if (a.active_mask) a.active_mask[ch] = support;
  if (a.status) {
    uint8_t st = 0;
    if (!converged) st |= CH_NNLS_MAXITER;
    if (!finite) st |= CH_NONFINITE;
    if (bad) st |= CH_BADINPUT;
    a.status[ch] = st;
  }
  if (a.iters) {
    const int fo = adds + adds64 < 4095 ? adds + adds64 : 4095;
    const int fi = solves < 4095 ? solves : 4095;
    a.iters[ch] = 1 | (fo << 8) | (fi << 20);
  }
}

template <int N, int K, bool WARM>
__device__ __forceinline__ void fit_channel(const MixedArgs& a, const DevMixed& T, int64_t ch, unsigned lanes) {
  double y[N], sig;
  const bool bad = whiten<N>(a, T, ch, y, sig);
  unsigned m = 0;
  float xw[K];
  if (WARM) {
    m = a.warm_mask[ch];
    const float* wa = a.warm_amp + ch * a.warm_stride;
#pragma unroll
    for (int k = 0; k < K; ++k) xw[k] = wa[k];
  }
  fit_from_y<N, K>(a, T, ch, y, sig, bad, WARM, m, xw, lanes);
}

// One launch per condition set: lanes of other sets stay idle (the
// persistent schedule groups channels by set instead). Out-of-range set
// indices are flagged by the first launch.
template <int N, int K>
__global__ void __launch_bounds__(128) fit_mixed_kernel(const MixedArgs a, int set, int flag_bad) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  bool mine = false;
  if (ch < a.n) {
    const int t = a.ctype ? int(a.ctype[ch]) : 0;
    if (t >= a.n_ctypes) {
      if (flag_bad) {
        if (a.status) a.status[ch] = CH_BADINPUT;
        a.chi2[ch] = 0.;
      }
    } else {
      mine = t == set && t != a.skip_set;
    }
  }
  const unsigned lanes = __ballot_sync(0xffffffffu, mine);  // taken while the warp is converged
  if (mine) fit_channel<N, K, false>(a, a.tab[set], ch, lanes);
}

// --------------------------------------------------------------------------
// Fused learned warm start: whitening -> MLP on the tensor cores -> warm fit
// --------------------------------------------------------------------------
struct FusedSmem {
  __nv_bfloat16 W1[MLP_H][MLP_IN + 8];
  __nv_bfloat16 W2[MLP_H][MLP_H + 8];
  __nv_bfloat16 W3[MLP_OUT][MLP_H + 8];
  float b1[MLP_H], b2[MLP_H], b3[MLP_OUT];
  __nv_bfloat16 X[128][MLP_IN + 8];
  float O[128][MLP_OUT + 1];
};

// Two adjacent n8 accumulator tiles (columns c0.. and c0+8..) after bias and
// GELU, packed as the BF16 A fragment of the next layer's k16 slice.
__device__ __forceinline__ void gelu_pack(const float (&c0)[4], const float (&c1)[4], const float* bias, int col0,
                                          uint32_t (&h)[4]) {
  h[0] = pack_bf16(gelu(c0[0] + bias[col0]), gelu(c0[1] + bias[col0 + 1]));
  h[1] = pack_bf16(gelu(c0[2] + bias[col0]), gelu(c0[3] + bias[col0 + 1]));
  h[2] = pack_bf16(gelu(c1[0] + bias[col0 + 8]), gelu(c1[1] + bias[col0 + 9]));
  h[3] = pack_bf16(gelu(c1[2] + bias[col0 + 8]), gelu(c1[3] + bias[col0 + 9]));
}

// The MLP of the warp's 32 channels (rows 32*warp.. of S.X) into S.O. The
// hidden activations stay in registers: the m16n8 accumulators of one layer,
// two n8 tiles at a time, are exactly the m16n8k16 A fragments of the next.
// Layer 2 is produced 16 columns at a time and each slice is folded into
// layer 3 at once, so only H1 is held (32 registers) and the code stays small.
__device__ __forceinline__ void warp_mlp(FusedSmem& S, int warp) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll 1
  for (int mt = 0; mt < 2; ++mt) {
    const int r = warp * 32 + mt * 16 + g;
    uint32_t a0[4];
    a0[0] = ld32(&S.X[r][2 * t]);
    a0[1] = ld32(&S.X[r + 8][2 * t]);
    a0[2] = ld32(&S.X[r][8 + 2 * t]);
    a0[3] = ld32(&S.X[r + 8][8 + 2 * t]);
    uint32_t h1[8][4];
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
      float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t b0[2] = {ld32(&S.W1[16 * kt + g][2 * t]), ld32(&S.W1[16 * kt + g][8 + 2 * t])};
      const uint32_t b1[2] = {ld32(&S.W1[16 * kt + 8 + g][2 * t]), ld32(&S.W1[16 * kt + 8 + g][8 + 2 * t])};
      mma_bf16(c0, a0, b0);
      mma_bf16(c1, a0, b1);
      gelu_pack(c0, c1, S.b1, 16 * kt + 2 * t, h1[kt]);
    }
    float o[4][4];
#pragma unroll
    for (int n3 = 0; n3 < 4; ++n3)
#pragma unroll
      for (int h = 0; h < 4; ++h) o[n3][h] = 0.f;
#pragma unroll 1
    for (int nt = 0; nt < 8; ++nt) {
      float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kt = 0; kt < 8; ++kt) {
        const uint32_t b0[2] = {ld32(&S.W2[16 * nt + g][16 * kt + 2 * t]),
                                ld32(&S.W2[16 * nt + g][16 * kt + 8 + 2 * t])};
        const uint32_t b1[2] = {ld32(&S.W2[16 * nt + 8 + g][16 * kt + 2 * t]),
                                ld32(&S.W2[16 * nt + 8 + g][16 * kt + 8 + 2 * t])};
        mma_bf16(c0, h1[kt], b0);
        mma_bf16(c1, h1[kt], b1);
      }
      uint32_t h2[4];
      gelu_pack(c0, c1, S.b2, 16 * nt + 2 * t, h2);
#pragma unroll
      for (int n3 = 0; n3 < 4; ++n3) {
        const uint32_t b3[2] = {ld32(&S.W3[8 * n3 + g][16 * nt + 2 * t]),
                                ld32(&S.W3[8 * n3 + g][16 * nt + 8 + 2 * t])};
        mma_bf16(o[n3], h2, b3);
      }
    }
#pragma unroll
    for (int n3 = 0; n3 < 4; ++n3) {
      const int c = 8 * n3 + 2 * t;
      S.O[r][c] = o[n3][0] + S.b3[c];
      S.O[r][c + 1] = o[n3][1] + S.b3[c + 1];
      S.O[r + 8][c] = o[n3][2] + S.b3[c];
      S.O[r + 8][c + 1] = o[n3][3] + S.b3[c + 1];
    }
  }
}

__global__ void __launch_bounds__(128, 3) fit_warm_fused_kernel(const MixedArgs a, const FusedMlp w) {
  extern __shared__ __align__(16) unsigned char fused_smem[];
  FusedSmem& S = *reinterpret_cast<FusedSmem*>(fused_smem);
  const int tid = threadIdx.x, warp = tid >> 5;
  const __nv_bfloat16* W1 = reinterpret_cast<const __nv_bfloat16*>(w.W1);
  const __nv_bfloat16* W2 = reinterpret_cast<const __nv_bfloat16*>(w.W2);
  const __nv_bfloat16* W3 = reinterpret_cast<const __nv_bfloat16*>(w.W3);
  for (int e = tid; e < MLP_H * MLP_IN; e += 128) S.W1[e / MLP_IN][e % MLP_IN] = W1[e];
  for (int e = tid; e < MLP_H * MLP_H; e += 128) S.W2[e / MLP_H][e % MLP_H] = W2[e];
  for (int e = tid; e < MLP_OUT * MLP_H; e += 128) S.W3[e / MLP_H][e % MLP_H] = W3[e];
  for (int e = tid; e < MLP_H; e += 128) {
    S.b1[e] = w.b1[e];
    S.b2[e] = w.b2[e];
  }
  for (int e = tid; e < MLP_OUT; e += 128) S.b3[e] = w.b3[e];
  __syncthreads();
  for (int64_t base = int64_t(blockIdx.x) * 128; base < a.n; base += int64_t(gridDim.x) * 128) {
    const int64_t ch = base + tid;
    const bool active = ch < a.n;
    const int ct = active ? (a.ctype ? int(a.ctype[ch]) : 0) : -1;
    const bool learned = active && ct == w.set;
    const unsigned lanes = __ballot_sync(0xffffffffu, learned);
    if (active && ct >= a.n_ctypes) {
      if (a.status) a.status[ch] = CH_BADINPUT;
      a.chi2[ch] = 0.;
    }
    double y[10], sig = 1.;
    bool bad = false;
    float f[MLP_IN], scale = 0.f;
#pragma unroll
    for (int j = 0; j < MLP_IN; ++j) f[j] = 0.f;
    if (learned) {
      bad = whiten<10>(a, a.tab[ct], ch, y, sig);
      mlp_features(y, sig, f, &scale);
    }
#pragma unroll
    for (int j = 0; j < MLP_IN; j += 2)
      *reinterpret_cast<uint32_t*>(&S.X[tid][j]) = pack_bf16(f[j], f[j + 1]);
    __syncwarp();
    warp_mlp(S, warp);
    __syncwarp();
    if (learned) {
      unsigned m = 0;
      float xw[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        if (S.O[tid][k] > 0.f && scale > 0.f) m |= 1u << k;
        xw[k] = softplusf(S.O[tid][10 + k]) * scale * w.inv_gnorm[k];
      }
      fit_from_y<10, 10>(a, a.tab[ct], ch, y, sig, bad, true, m, xw, lanes);
    }
    // channels of other condition sets are fitted by a cold launch that skips this set
    __syncwarp();
  }
}

}  // namespace

cudaError_t launch_fit_warm_fused(const MixedArgs& a, const FusedMlp& w, int sms, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  static bool attr_set = false;
  const size_t smem = sizeof(FusedSmem);
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(fit_warm_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int64_t tiles = (a.n + 127) / 128;
  const int64_t cap = int64_t(sms) * 3;
  const int grid = int(tiles < cap ? tiles : cap);
  fit_warm_fused_kernel<<<grid, 128, smem, s>>>(a, w);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || a.n_ctypes == 1 || !a.ctype) return e;
  MixedArgs rest = a;  // channels of the other condition sets: cold mixed fit
  rest.skip_set = w.set;
  return launch_fit_mixed(rest, 128, s);
}

cudaError_t launch_fit_mixed(const MixedArgs& a, int block, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  const unsigned grid = unsigned((a.n + block - 1) / block);
  int flag_bad = 1;
  for (int t = 0; t < a.n_ctypes; ++t) {
    if (t == a.skip_set) continue;
    const DevMixed& T = a.tab[t];
    if (T.N == 10 && T.K == 10) fit_mixed_kernel<10, 10><<<grid, block, 0, s>>>(a, t, flag_bad);
    else if (T.N == 8 && T.K == 8) fit_mixed_kernel<8, 8><<<grid, block, 0, s>>>(a, t, flag_bad);
    else return cudaErrorInvalidValue;
    flag_bad = 0;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace mfgb
