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

namespace mfgb {
namespace {

template <int N, int K>
struct ChannelFP {
  double y[N];
  float y32[N];
  float c32[K];
  float x32[K];
  double x64[K];
};

template <int N, int K>
__device__ __forceinline__ void solve32(const DevMixed& T, unsigned m, const float* y32, float* s) {
  const float* P = T.pinv32 + T.offset[m];
  int r = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    s[k] = 0.f;
    if (m & (1u << k)) {
      float acc = 0.f;
#pragma unroll
      for (int i = 0; i < N; ++i) acc = fmaf(__ldg(P + r * N + i), y32[i], acc);
      s[k] = acc;
      ++r;
    }
  }
}

template <int N, int K>
__device__ __forceinline__ void solve64(const DevMixed& T, unsigned m, const double* y, double* s) {
  const double* P = T.pinv64 + T.offset[m];
  int r = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    s[k] = 0.;
    if (m & (1u << k)) {
      double acc = 0.;
#pragma unroll
      for (int i = 0; i < N; ++i) acc = fma(__ldg(P + r * N + i), y[i], acc);
      s[k] = acc;
      ++r;
    }
  }
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

template <int N, int K, bool WARM>
__device__ void fit_channel(const MixedArgs& a, const DevMixed& T, int64_t ch) {
  const double* in = a.samples + ch * a.sample_stride;
  const double sig = a.pederr[ch];
  double s[N];
  bool bad = !isfinite(sig) || !(sig > 0.);
#pragma unroll
  for (int i = 0; i < N; ++i) {
    s[i] = in[i];
    bad = bad || !isfinite(s[i]);
  }
  // 1. whitening with the shared inverse factor
  double y[N];
  float y32[N];
  float ynorm2 = 0.f;
  {
    int w = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double acc = 0.;
#pragma unroll
      for (int j = 0; j <= i; ++j) acc = fma(T.W64[w + j], s[j], acc);
      w += i + 1;
      y[i] = acc;
      y32[i] = float(acc);
      ynorm2 = fmaf(y32[i], y32[i], ynorm2);
    }
  }
  // 2. FP32 active-set search
  float c32[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) acc = fmaf(T.G32[k * N + i], y32[i], acc);
    c32[k] = acc;
  }
  const float ynorm = sqrtf(ynorm2);
  const unsigned full = (1u << K) - 1u;
  unsigned m = 0;
  float x32[K];
#pragma unroll
  for (int k = 0; k < K; ++k) x32[k] = 0.f;
  int adds = 0, solves = 0;
  auto s32 = [&](unsigned mm, float* out) { solve32<N, K>(T, mm, y32, out); };
  if (WARM) {
    m = unsigned(a.warm_mask[ch]) & full;
    const float* wa = a.warm_amp + ch * a.warm_stride;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (m & (1u << k)) x32[k] = fmaxf(wa[k], 1e-30f);
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
  // 3. FP64 judge: continue the same loop in FP64 from the FP32 passive set
  double x[K];
#pragma unroll
  for (int k = 0; k < K; ++k) x[k] = double(x32[k]);
  auto s64 = [&](unsigned mm, double* out) { solve64<N, K>(T, mm, y, out); };
  if (m) solves += inner_loop<K>(m, x, s64);
  double c64[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double acc = 0.;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) acc = fma(T.G64[k * N + i], y[i], acc);
    c64[k] = acc;
  }
  const double tol64 = a.eps * sig * sig;
  bool converged = false;
  int adds64 = 0;
  for (int it = 0; it < a.max_iter64; ++it) {
    double wmax = 0.;
    int imax = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (m & (1u << k)) continue;
      double acc = c64[k];
#pragma unroll
      for (int j = 0; j < K; ++j)
        if (m & (1u << j)) acc = fma(-T.H64[k * KMAX + j], x[j], acc);
      if (imax < 0 || acc > wmax) {
        wmax = acc;
        imax = k;
      }
    }
    if (imax < 0 || !(wmax >= tol64)) {
      converged = true;
      break;
    }
    m |= 1u << imax;
    ++adds64;
    solves += inner_loop<K>(m, x, s64);
  }
  // 4. chi2 in FP64
  double chi2 = 0.;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double acc = y[i];
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (i >= T.gfz[k]) acc = fma(-T.G64[k * N + i], x[k], acc);
    chi2 = fma(acc, acc, chi2);
  }
  chi2 = chi2 / (sig * sig);

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

template <bool WARM>
__global__ void __launch_bounds__(128) fit_mixed_kernel(const MixedArgs a) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (ch >= a.n) return;
  const int t = a.ctype ? int(a.ctype[ch]) : 0;
  if (t >= a.n_ctypes) {
    if (a.status) a.status[ch] = CH_BADINPUT;
    a.chi2[ch] = 0.;
    return;
  }
  const DevMixed& T = a.tab[t];
  if (T.N == 10 && T.K == 10) fit_channel<10, 10, WARM>(a, T, ch);
  else if (T.N == 8 && T.K == 8) fit_channel<8, 8, WARM>(a, T, ch);
  else if (a.status) a.status[ch] = CH_BADINPUT;  // shapes without a mixed build (rejected on the host)
}

}  // namespace

cudaError_t launch_fit_mixed(const MixedArgs& a, int block, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  const int64_t grid = (a.n + block - 1) / block;
  if (a.warm_mask) fit_mixed_kernel<true><<<unsigned(grid), block, 0, s>>>(a);
  else fit_mixed_kernel<false><<<unsigned(grid), block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mfgb
