// Device code shared by the grid (fit_mixed.cu) and persistent (fit_sched.cu)
// schedules of the mixed-precision multifit: the passive-set solves from the
// operator tables, the FNNLS inner loop, and the per-channel bodies of the FP32
// search, the FP64 judge and the FP64 repair. Both schedules run the same
// per-channel arithmetic, so their results are identical.
#pragma once
#include <cfloat>

#include "mf_internal.h"

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

// The same solve without branches: every lane computes all K rows, rows of
// columns outside the set read the table's zero row. On this GPU an FP64 warp
// instruction costs the full pipe time whatever the number of active lanes, so
// the FP64 judge keeps all 32 lanes busy on every instruction.
template <int N, int K>
__device__ __forceinline__ void solve64_dense(const DevMixed& T, unsigned m, const double* y, double* s) {
  const double* P = T.pinv64 + __ldg(T.offset + m);
  const double* Z = T.pinv64 + T.zero_row;
  int r = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const bool in = (m >> k) & 1u;
    const double2* row = reinterpret_cast<const double2*>(in ? P + r * N : Z);
    r += in ? 1 : 0;
    double acc = 0.;
#pragma unroll
    for (int q = 0; q < N / 2; ++q) {
      const double2 v = __ldg(row + q);
      acc = fma(v.x, y[2 * q], acc);
      acc = fma(v.y, y[2 * q + 1], acc);
    }
    s[k] = acc;
  }
}

// Appends value to a queue (one atomic per warp for the lanes appending together).
__device__ __forceinline__ void enqueue(unsigned* count, int* queue, int value) {
  const unsigned act = __activemask();
  const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(count, unsigned(__popc(act)));
  base = __shfl_sync(act, base, leader);
  queue[base + __popc(act & ((1u << lane) - 1u))] = value;
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

// c = G^T y in FP32 and sum_i |G_ik y_i| (its rounding-error scale)
template <int N, int K>
__device__ __forceinline__ void gram_rhs32(const DevMixed& T, const float* y32, float* c, float* cmag) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float acc = 0.f, mag = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      acc = fmaf(T.G32[k * N + i], y32[i], acc);
      mag = fmaf(fabsf(T.G32[k * N + i]), fabsf(y32[i]), mag);
    }
    c[k] = acc;
    if (cmag) cmag[k] = mag;
  }
}

// ---------------------------------------------------------------------------
// Double-float arithmetic for the search's KKT screen
// ---------------------------------------------------------------------------
// The FP32 search's gradient c - H x is as accurate as the FP32 solution x,
// whose error is the FP32 table's rounding amplified by cond(G_S) (~5e4 for
// ECAL), and no FP32 residual y - G x resolves a ~1e4 signal to its ~1 noise.
// The screen below therefore forms y and the residual in double-float (a
// value is an unevaluated sum hi + lo of two floats) with the error-free
// transforms of Dekker (TwoProduct via FMA) and Knuth (TwoSum), all in FP32.
// The _rn intrinsics keep the compiler from contracting the transforms.
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = fmaf(a, b, -p);
}

// (hi, lo) += (p, e), renormalised.
__device__ __forceinline__ void df_acc(float& hi, float& lo, float p, float e) {
  const float s = __fadd_rn(hi, p);
  const float v = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, v)), __fsub_rn(p, v));
  const float t = __fadd_rn(__fadd_rn(err, lo), e);
  hi = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(hi, s));
}

// A double as hi + lo without FP64 arithmetic: hi = its top 24 significand
// bits (truncation), lo = the next 29 bits rounded to 24 (2^-47 relative in
// all). Values below 2^-74 or above 2^127 keep hi alone.
__device__ __forceinline__ void split64(double v, float& hi, float& lo) {
  hi = __double2float_rz(v);
  const long long b = __double_as_longlong(v);
  const int ex = int((b >> 52) & 0x7ff);
  lo = 0.f;
  if (ex >= 949 && ex <= 1150) {
    const float scale = __int_as_float((ex - 1075 + 127) << 23);  // 2^(ex - 1023 - 52)
    lo = float(int(b & 0x1fffffffLL)) * scale;
    if (b < 0) lo = -lo;
  }
}

// The residual r = L_R^-1 (s - P x) of amplitudes x: u = s - P x in
// double-float (s = sh + sl, P = P32 + P32lo, x exact floats; column by column,
// so the N row chains interleave), then rounded to FP32 -- u is at the noise
// level, so the FP32 whitening that follows adds only 2^-24 cond(L_R) relative
// error (cond(L_R) = 5.7 for the ECAL correlation rho = 0.7).
template <int N, int K>
__device__ __forceinline__ void residual_df(const DevMixed& T, const float* sh, const float* sl, const float* x,
                                            float* r) {
  float uh[N], ul[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    uh[i] = sh[i];
    ul[i] = sl[i];
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const float xk = -x[k];
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) {  // P and G share their structural zeros (L_R^-1 is lower triangular)
        float p, e;
        two_prod(T.P32[k * N + i], xk, p, e);
        e = fmaf(T.P32lo[k * N + i], xk, e);
        df_acc(uh[i], ul[i], p, e);
      }
  }
  float u[N];
#pragma unroll
  for (int i = 0; i < N; ++i) u[i] = __fadd_rn(uh[i], ul[i]);
  int w = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j <= i; ++j) acc = fmaf(T.W32[w + j], u[j], acc);
    w += i + 1;
    r[i] = acc;
  }
}

// The KKT screen of the FP32 search's set (its own kernel between the search
// and the judge: convergent, on the FP32 pipe, no data-dependent loop): the
// accurate residual of the FP32 solution (residual_df), two refinement steps
// of x on the passive set through the FP32 table (each shrinks the table's
// error by about cond(G_S) 2^-24), the gradient w = G^T r of every column
// outside the set; returns the mask of the columns whose gradient is
// provably positive (w_k > 2^-16 sum_i |G_ik r_i|, a bound well above the
// refined gradient's error) and leaves the refined amplitudes in x32 where
// they stay feasible. solve_rhs(m, rhs, out) is the set's table solve on rhs.
template <int N, int K, typename SolveRhs>
__device__ __forceinline__ unsigned refine_screen(const DevMixed& T, const float* sh, const float* sl, unsigned m,
                                                  float* x32, int& solves, SolveRhs solve_rhs) {
  float xr[K], r[N], d[K];
#pragma unroll
  for (int k = 0; k < K; ++k) xr[k] = x32[k];
  residual_df<N, K>(T, sh, sl, xr, r);
#pragma unroll
  for (int step = 0; step < 2; ++step) {
    solve_rhs(m, r, d);
#pragma unroll
    for (int k = 0; k < K; ++k) xr[k] += d[k];
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int i = 0; i < N; ++i)
        if (i >= T.gfz[k]) r[i] = fmaf(-T.G32[k * N + i], d[k], r[i]);
  }
  solves += 2;
  // the refined amplitudes replace the search's where they stay feasible
  bool feasible = true;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if ((m & (1u << k)) && !(xr[k] > 0.f)) feasible = false;
  if (feasible) {
#pragma unroll
    for (int k = 0; k < K; ++k) x32[k] = xr[k];
  }
  unsigned add = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float w = 0.f, mag = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) {
        w = fmaf(T.G32[k * N + i], r[i], w);
        mag = fmaf(fabsf(T.G32[k * N + i]), fabsf(r[i]), mag);
      }
    if (!(m & (1u << k)) && w > 0x1p-16f * mag) add |= 1u << k;
  }
  return add;
}

// ---------------------------------------------------------------------------
// FP32 active-set search
// ---------------------------------------------------------------------------
// Outer iterations of the search from a learned warm start. Nearly every
// channel settles within two; the rare channel that keeps adding columns held
// its whole warp, and after two iterations it is left to the judge, which
// queues it for the fix (and, failing that, the repair) in full warps.
// Measured on 10M warm channels: search 1.42 -> 1.00 ms (cap 4: 1.03, cap 1:
// 0.93 with the queues 0.04 ms longer), same KKT points. Cold starts keep
// max_iter32.
constexpr int kWarmSearchIters = 2;
// The FP32 search of channel ch (one lane): writes the hand-off (passive mask,
// add and solve counts, FP32 amplitudes) for the FP64 judge.
template <int N, int K, bool WARM>
__device__ __forceinline__ void search_body(const MixedArgs& a, const DevMixed& T, int64_t ch) {
  const double* in = a.samples + ch * a.sample_stride;
  float sf[N], y32[N], ynorm2 = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i) sf[i] = float(in[i]);
  {
    int w = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      float acc = 0.f;
#pragma unroll
      for (int j = 0; j <= i; ++j) acc = fmaf(T.W32[w + j], sf[j], acc);
      w += i + 1;
      y32[i] = acc;
      ynorm2 = fmaf(acc, acc, ynorm2);
    }
  }
  float c32[K];
  gram_rhs32<N, K>(T, y32, c32, nullptr);
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
  const int iters = WARM ? kWarmSearchIters : a.max_iter32;
  for (int it = 0; it < iters; ++it) {
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
  a.ws_mask[ch] = uint16_t(m);
  a.ws_count[ch] = uint16_t((adds < 255 ? adds : 255) | ((solves < 255 ? solves : 255) << 8));
  float* wx = a.ws_x + ch * K;
#pragma unroll
  for (int k = 0; k < K; ++k) wx[k] = x32[k];
}

// ---------------------------------------------------------------------------
// FP64 judge
// ---------------------------------------------------------------------------

// FP64 residual r = y - G x (dense; G's structural zeros are skipped
// uniformly) and the index and value of the largest gradient w = G^T r over
// the columns outside the passive set m (and, with viol, the mask of those at
// or above tol).
template <int N, int K>
__device__ __forceinline__ void residual_gradient(const DevMixed& T, const double* y, const double* x, unsigned m,
                                                  double* r, double& wmax, int& imax, double tol = 0.,
                                                  unsigned* viol = nullptr) {
#pragma unroll
  for (int i = 0; i < N; ++i) r[i] = y[i];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) r[i] = fma(-T.G64[k * N + i], x[k], r[i]);
  wmax = 0.;
  imax = -1;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double w = 0.;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) w = fma(T.G64[k * N + i], r[i], w);
    const bool cand = !(m & (1u << k)) && (imax < 0 || w > wmax);
    wmax = cand ? w : wmax;
    imax = cand ? k : imax;
    if (viol && !(m & (1u << k)) && w >= tol) *viol |= 1u << k;
  }
}

// y = L_R^-1 s in FP64 (packed rows, no division); returns true for a
// non-finite or non-positive input.
template <int N>
__device__ __forceinline__ bool whiten64(const MixedArgs& a, const DevMixed& T, int64_t ch, double* y, double& sig) {
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

// Outputs of a judged channel: amplitudes, chi2, in-time amplitude, active
// mask (support of x), status, counters, FP64 flops.
// A finite double, decided on its exponent bits (no FP64 instruction).
__device__ __forceinline__ bool finite64(double v) {
  return ((__double2hiint(v) >> 20) & 0x7ff) != 0x7ff;
}

template <int N, int K>
__device__ __forceinline__ void store_outputs(const MixedArgs& a, const DevMixed& T, int64_t ch, const double* x,
                                              double chi2, bool bad, bool converged, int adds, int solves, int f64) {
  double* out = a.amplitudes + ch * a.amp_stride;
  bool finite = finite64(chi2);
  uint16_t support = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    out[k] = x[k];
    finite = finite && finite64(x[k]);
    if (pos64(x[k])) support |= uint16_t(1u << k);
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
    const int fo = adds < 4095 ? adds : 4095;
    const int fi = solves < 4095 ? solves : 4095;
    a.iters[ch] = 1 | (fo << 8) | (fi << 20);
  }
  if (a.flops) a.flops[ch] = double(f64);
}

// The same with chi2 = ||r||^2 / pederr^2 from the FP64 residual.
template <int N, int K>
__device__ __forceinline__ void write_outputs(const MixedArgs& a, const DevMixed& T, int64_t ch, const double* x,
                                              const double* r, double sig, bool bad, bool converged, int adds,
                                              int solves, int f64) {
  double chi2 = 0.;
#pragma unroll
  for (int i = 0; i < N; ++i) chi2 = fma(r[i], r[i], chi2);
  chi2 = chi2 / (sig * sig);
  store_outputs<N, K>(a, T, ch, x, chi2, bad, converged, adds, solves, f64 + 2 * N + 2);
}

// The repair path (the FP64 solve on the FP32 set has a non-positive
// component, or the FP64 KKT test fails), self-contained: the FNNLS loop in
// FP64 from the FP32 passive set and the feasible FP32 amplitudes, to the FP64
// KKT point; writes the channel's outputs.
template <int N, int K>
__device__ __forceinline__ void judge_repair(const MixedArgs& a, const DevMixed& T, int64_t ch) {
  double y[N], sig;
  const bool bad = whiten64<N>(a, T, ch, y, sig);
  unsigned m = a.ws_mask[ch];
  const unsigned cnt = a.ws_count[ch];
  int adds = int(cnt & 255u), solves = int(cnt >> 8) + 1;
  int f64 = N * (N + 1) + 4 * N * K;  // the judge's attempt
  auto s64 = [&](unsigned mm, double* out) {
    solve64_dense<N, K>(T, mm, y, out);
    f64 += 2 * N * K;
  };
  double x[K], r[N];
  const float* wx = a.ws_x + ch * K;
#pragma unroll
  for (int k = 0; k < K; ++k) x[k] = double(wx[k]);
  solves += inner_loop<K>(m, x, s64);
  const double tol64 = a.eps * sig * sig;
  bool converged = false;
  double wmax;
  int imax;
  for (int it = 0; it < a.max_iter64; ++it) {
    unsigned viol = 0;
    residual_gradient<N, K>(T, y, x, m, r, wmax, imax, tol64, &viol);
    f64 += 4 * N * K;
    if (viol == 0u) {
      converged = true;
      break;
    }
    // add every violating column at once (the KKT point of this strictly
    // convex problem is unique, so the order of additions does not matter)
    m |= viol;
    adds += __popc(viol);
    solves += inner_loop<K>(m, x, s64);
  }
  if (!converged) residual_gradient<N, K>(T, y, x, m, r, wmax, imax);  // residual of the last state
  write_outputs<N, K>(a, T, ch, x, r, sig, bad, converged, adds, solves, f64);
}

// The KKT screen of channel ch (one lane, FP32, branch-free), run on cold
// starts before the judge: refines the search's amplitudes on its set and,
// when columns provably violate the KKT condition, queues the channel for
// fix_body (ws_fixq, the columns to add in ws_add).
template <int N, int K>
__device__ __forceinline__ void screen_body(const MixedArgs& a, const DevMixed& T, int64_t ch, unsigned* fix_count) {
  const unsigned m = a.ws_mask[ch];
  float x32[K];
  float* wx = a.ws_x + ch * K;
#pragma unroll
  for (int k = 0; k < K; ++k) x32[k] = wx[k];
  const double* in = a.samples + ch * a.sample_stride;
  float sh[N], sl[N];
#pragma unroll
  for (int i = 0; i < N; ++i) split64(in[i], sh[i], sl[i]);
  int solves = 0;
  const unsigned add = refine_screen<N, K>(T, sh, sl, m, x32, solves,
                                           [&](unsigned mm, const float* rhs, float* out) { solve32<N, K>(T, mm, rhs, out); });
#pragma unroll
  for (int k = 0; k < K; ++k) wx[k] = x32[k];
  if (add) {
    a.ws_add[ch] = uint16_t(add);
    enqueue(fix_count, a.ws_fixq, int(ch));
  }
}

// A channel queued for fixing by the screen or the judge (entry = the
// channel's index in the chunk; ws_add[ch] = the columns that provably
// violate the KKT condition):
// the FNNLS step with the added columns in FP32 (the inner loop drops those
// that come out non-positive), then, with rounds = 2, the double-float screen
// of the new set and, if it finds more, one more step. Writes the hand-off for
// the judge. Cold starts (queued by the screen, judged once after) take two
// rounds; warm starts (queued by the judge, judged again after) one: there the
// screen round cost more than the repairs it saved (warm step 6.31 -> 6.14 ms
// per 10M with one round; cold with one round 9.5 -> 13.0 ms, repairs x9).
template <int N, int K>
__device__ __forceinline__ void fix_body(const MixedArgs& a, const DevMixed& T, unsigned entry, int rounds) {
  const int64_t ch = int64_t(entry);
  unsigned add = a.ws_add[ch];
  unsigned m = a.ws_mask[ch];
  const unsigned cnt = a.ws_count[ch];
  int adds = int(cnt & 255u), solves = int(cnt >> 8);
  float x32[K];
  float* wx = a.ws_x + ch * K;
#pragma unroll
  for (int k = 0; k < K; ++k) x32[k] = wx[k];
  const double* in = a.samples + ch * a.sample_stride;
  float sh[N], sl[N], y32[N];
#pragma unroll
  for (int i = 0; i < N; ++i) split64(in[i], sh[i], sl[i]);
  {
    int w = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      float acc = 0.f;
#pragma unroll
      for (int j = 0; j <= i; ++j) acc = fmaf(T.W32[w + j], sh[j], acc);
      w += i + 1;
      y32[i] = acc;
    }
  }
  auto s32 = [&](unsigned mm, float* out) { solve32<N, K>(T, mm, y32, out); };
  auto srhs = [&](unsigned mm, const float* rhs, float* out) { solve32<N, K>(T, mm, rhs, out); };
#pragma unroll 1
  for (int round = 0; round < 2 && add; ++round) {
    m |= add;
    adds += __popc(add);
    solves += inner_loop<K>(m, x32, s32);
    add = round + 1 < rounds ? refine_screen<N, K>(T, sh, sl, m, x32, solves, srhs) : 0u;
  }
  a.ws_mask[ch] = uint16_t(m);
  a.ws_count[ch] = uint16_t((adds < 255 ? adds : 255) | ((solves < 255 ? solves : 255) << 8));
#pragma unroll
  for (int k = 0; k < K; ++k) wx[k] = x32[k];
}

// The FP32 screen of the KKT test on the FP64 residual r: the FP32 gradient
// w_k = G_k^T r of a column outside m is accurate to (N + 2) 2^-24 sum_i
// |G_ik r_i| < 2^-19 sum (N <= 10 rounded FMAs, plus the rounding of G and r
// to FP32); a column passes only if w_k plus that bound stays below tol, so
// every column the FP64 test w_k >= tol could flag is sent to the FP64
// repair, and only columns within that bound of tol are sent there
// needlessly. Returns true when no column needs the FP64 test; add collects
// the columns that provably violate it.
template <int N, int K>
__device__ __forceinline__ bool kkt_screen32(const DevMixed& T, const double* r, unsigned m, float tol,
                                             unsigned& add) {
  float rf[N];
#pragma unroll
  for (int i = 0; i < N; ++i) rf[i] = float(r[i]);
  bool ok = true;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float w = 0.f, mag = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i >= T.gfz[k]) {
        w = fmaf(T.G32[k * N + i], rf[i], w);
        mag = fmaf(fabsf(T.G32[k * N + i]), fabsf(rf[i]), mag);
      }
    if (!(m & (1u << k)) && !(fmaf(0x1p-19f, mag, w) < tol)) ok = false;
    if (!(m & (1u << k)) && fmaf(-0x1p-19f, mag, w) > tol) add |= 1u << k;  // provably violating
  }
  return ok;
}

// The FP64 judge of channel ch (one lane): writes the outputs; or, when
// columns provably violate the KKT condition and the amplitudes are positive
// and fix_count is given, queues the channel for the FP32 fix (ws_fixq,
// the columns to add in ws_add); otherwise queues it for the FP64 repair (ws_queue).
// The FP64 solve on the search's passive set and the residual run column by
// column over the set only (each lane its own trip count; a warp runs as many
// iterations as its largest set): x_k = G_S^+_k y from the FP64 table, then
// r -= G_k x_k at once, with G_k read from global memory (a different column
// in every lane). The columns outside the set, once run through a zero row,
// were exact no-ops. The amplitudes are written as they come; a channel the
// judge queues gets them rewritten by the fix or the repair.
template <int N, int K>
__device__ __forceinline__ void judge_body(const MixedArgs& a, const DevMixed& T, int64_t ch, unsigned* qcount,
                                           unsigned* fix_count) {
  const unsigned m = a.ws_mask[ch];
  const unsigned cnt = a.ws_count[ch];
  double y[N], sig;
  const bool bad = whiten64<N>(a, T, ch, y, sig);
  double r[N];
#pragma unroll
  for (int i = 0; i < N; ++i) r[i] = y[i];
  bool ok = true, finite = true;
  uint16_t support = 0;
  double xin = 0.;
  double* out = a.amplitudes + ch * a.amp_stride;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (!((m >> k) & 1u)) out[k] = 0.;
  const int p = __popc(m);
  {
    const double* P = T.pinv64 + __ldg(T.offset + m);
    unsigned rest = m;
#pragma unroll 1
    for (int rr = 0; rr < p; ++rr) {
      const int k = __ffs(rest) - 1;
      rest &= rest - 1u;
      const double2* row = reinterpret_cast<const double2*>(P + rr * N);
      double xk = 0.;
#pragma unroll
      for (int q = 0; q < N / 2; ++q) {
        const double2 v = __ldg(row + q);
        xk = fma(v.x, y[2 * q], xk);
        xk = fma(v.y, y[2 * q + 1], xk);
      }
      if (!pos64(xk)) ok = false;
      const double2* g = reinterpret_cast<const double2*>(T.g64 + k * N);
#pragma unroll
      for (int q = 0; q < N / 2; ++q) {
        const double2 v = __ldg(g + q);
        r[2 * q] = fma(-v.x, xk, r[2 * q]);
        r[2 * q + 1] = fma(-v.y, xk, r[2 * q + 1]);
      }
      out[k] = xk;
      finite = finite && finite64(xk);
      if (pos64(xk)) support |= uint16_t(1u << k);
      if (k == T.intime_col) xin = xk;
    }
  }
  unsigned add = 0;
  const bool pos_ok = ok;
  if (ok) ok = kkt_screen32<N, K>(T, r, m, float(a.eps * sig * sig), add);
  if (!ok) {  // compaction into the fix or the repair queue
    if (fix_count && pos_ok && add) {
      a.ws_add[ch] = uint16_t(add);
      enqueue(fix_count, a.ws_fixq, int(ch));
    } else {
      enqueue(qcount, a.ws_queue, int(ch));
    }
    return;
  }
  double chi2 = 0.;
#pragma unroll
  for (int i = 0; i < N; ++i) chi2 = fma(r[i], r[i], chi2);
  chi2 = chi2 / (sig * sig);
  for (int k = K; k < a.amp_stride && k < KMAX; ++k) out[k] = 0.;
  a.chi2[ch] = chi2;
  if (a.intime) a.intime[ch] = T.intime_col >= 0 ? xin : 0.;
  if (a.active_mask) a.active_mask[ch] = support;
  if (a.status) {
    uint8_t st = 0;
    if (!(finite && finite64(chi2))) st |= CH_NONFINITE;
    if (bad) st |= CH_BADINPUT;
    a.status[ch] = st;
  }
  if (a.iters) {
    const int adds = int(cnt & 255u), solves = int(cnt >> 8) + 1;
    a.iters[ch] = 1 | ((adds < 4095 ? adds : 4095) << 8) | ((solves < 4095 ? solves : 4095) << 20);
  }
  // executed FP64 flops: whitening, the passive solve and residual (2N each per column), chi2
  if (a.flops) a.flops[ch] = double(N * (N + 1) + 4 * N * p + 2 * N + 2);
}

// ---------------------------------------------------------------------------
// The judge in double-float FP32 arithmetic (MF_PREC_FP32)
// ---------------------------------------------------------------------------
// The FP64 judge's steps -- y = L_R^-1 s, the solve x = G_S^+ y from the
// operator table, the residual r = y - G x, chi2 -- with every value an
// unevaluated float pair (hi + lo) and every product and sum through the
// error-free transforms above: ~2^-48 relative per operation against FP64's
// 2^-53, so amplitudes keep ~cond(G_S) 2^-48 (< 1e-9) relative accuracy. An
// emulated FMA costs ~17 FP32 flops, but on this GPU the FP32 pipe is ~64x
// the FP64 pipe. The KKT test is the FP64 judge's (FP32 screen with the
// 2^-19 rounding bound); rejected channels go to the same FP64 repair.

// acc += (ah + al) (bh + bl), dropping al * bl (2^-48 relative).
__device__ __forceinline__ void df_fma(float& hi, float& lo, float ah, float al, float bh, float bl) {
  float p, e;
  two_prod(ah, bh, p, e);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  df_acc(hi, lo, p, e);
}


template <int N, int K>
__device__ __forceinline__ void judge_df_body(const MixedArgs& a, const DevMixed& T, int64_t ch, unsigned* qcount,
                                              unsigned* fix_count) {
  const unsigned m = a.ws_mask[ch];
  const unsigned cnt = a.ws_count[ch];
  const double* in = a.samples + ch * a.sample_stride;
  const double sig = a.pederr[ch];
  bool bad = !finite64(sig) || !pos64(sig);
  float sgh, sgl;  // pederr as a float pair, its square as another
  split64(sig, sgh, sgl);
  float s2h, s2l;
  two_prod(sgh, sgh, s2h, s2l);
  s2l = fmaf(2.f * sgh, sgl, s2l);
  float sh[N], sl[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    bad = bad || !finite64(in[i]);
    split64(in[i], sh[i], sl[i]);
  }
  // y = L_R^-1 s
  float yh[N], yl[N];
  {
    int w = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      float hi = 0.f, lo = 0.f;
#pragma unroll
      for (int j = 0; j <= i; ++j) df_fma(hi, lo, T.W32[w + j], T.W32lo[w + j], sh[j], sl[j]);
      w += i + 1;
      yh[i] = hi;
      yl[i] = lo;
    }
  }
  // Column by column over the channel's passive set (its own trip count: a
  // warp runs as many iterations as its largest set, where a loop over all K
  // columns ran the inactive ones through a zero row as exact no-ops):
  // x_k = G_S^+_k y through the table's float pairs, dx_k = sum_i |G^+_ki y_i|
  // (the scale of x_k's round-off), then x_k enters the residual r = y - G x
  // at once. The loop stays rolled: unrolled, the judge's body ran to ~6,000
  // instructions and instruction fetch was its first stall. The amplitudes are
  // written as they come; a channel the judge queues gets them rewritten by
  // the fix or the repair.
  //
  // Round-off bounds, per channel. The table and y are exact to ~2^-48 and each
  // double-float multiply-add errs by ~2^-48 of its terms, so with N <= 10
  // terms per sum |x_k - x_S,k| <= N 2^-48 dx_k < 2^-44 dx_k (xb), and the
  // computed residual errs by at most e_i = sum_k |G_ik| (xb_k + 2^-44 |x_k|)
  // + 2^-44 |y_i| (the solve's error carried through G, plus the residual's
  // own rounding), so a gradient errs by at most sum_i |G_ik| e_i. Where the
  // true residual is tiny (near-exact fits, e.g. ten active pulses on ten
  // samples) these errors can flip the sign of a gradient or an amplitude, so
  // decisions inside the bounds go to the FP64 repair.
  float rh[N], rl[N], e[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    rh[i] = yh[i];
    rl[i] = yl[i];
    e[i] = 0x1p-44f * fabsf(yh[i]);
  }
  bool ok = true, finite = true;
  uint16_t support = 0;
  double xin = 0.;
  double* out = a.amplitudes + ch * a.amp_stride;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (!((m >> k) & 1u)) out[k] = 0.;
  {
    const int off = __ldg(T.offset + m);
    const int p = __popc(m);
    unsigned rest = m;
#pragma unroll 1
    for (int r = 0; r < p; ++r) {
      const int k = __ffs(rest) - 1;
      rest &= rest - 1u;
      const int row = off + r * N;
      float hi = 0.f, lo = 0.f, mag = 0.f;
      if constexpr (N % 2 == 0) {
        const float4* rp = reinterpret_cast<const float4*>(T.pinv2 + 2 * row);
#pragma unroll
        for (int i = 0; i < N; i += 2) {
          const float4 q = __ldg(rp + i / 2);
          df_fma(hi, lo, q.x, q.y, yh[i], yl[i]);
          mag = fmaf(fabsf(q.x), fabsf(yh[i]), mag);
          df_fma(hi, lo, q.z, q.w, yh[i + 1], yl[i + 1]);
          mag = fmaf(fabsf(q.z), fabsf(yh[i + 1]), mag);
        }
      } else {
        const float2* rp = reinterpret_cast<const float2*>(T.pinv2 + 2 * row);
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const float2 q = __ldg(rp + i);
          df_fma(hi, lo, q.x, q.y, yh[i], yl[i]);
          mag = fmaf(fabsf(q.x), fabsf(yh[i]), mag);
        }
      }
      const float xb = 0x1p-44f * mag;
      if (!(hi > xb)) ok = false;
      const float ek = fmaf(0x1p-44f, fabsf(hi), xb);
      // r -= G_k x_k (G's structural zeros add exact zeros)
      const float nh = -hi, nl = -lo;
      if constexpr (N % 2 == 0) {
        const float4* gp = reinterpret_cast<const float4*>(T.g2 + 2 * k * N);
#pragma unroll
        for (int i = 0; i < N; i += 2) {
          const float4 g = __ldg(gp + i / 2);
          df_fma(rh[i], rl[i], g.x, g.y, nh, nl);
          e[i] = fmaf(fabsf(g.x), ek, e[i]);
          df_fma(rh[i + 1], rl[i + 1], g.z, g.w, nh, nl);
          e[i + 1] = fmaf(fabsf(g.z), ek, e[i + 1]);
        }
      } else {
        const float2* gp = reinterpret_cast<const float2*>(T.g2 + 2 * k * N);
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const float2 g = __ldg(gp + i);
          df_fma(rh[i], rl[i], g.x, g.y, nh, nl);
          e[i] = fmaf(fabsf(g.x), ek, e[i]);
        }
      }
      const double xk = double(hi) + double(lo);
      out[k] = xk;
      finite = finite && finite64(xk);
      if (pos64(xk)) support |= uint16_t(1u << k);
      if (k == T.intime_col) xin = xk;
    }
  }
  const bool pos_ok = ok;
  unsigned add = 0;
  float rf[N];
#pragma unroll
  for (int i = 0; i < N; ++i) rf[i] = __fadd_rn(rh[i], rl[i]);
  if (ok) {
    const float tol = a.eps32 * s2h;
#pragma unroll 1
    for (int k = 0; k < K; ++k) {
      if (m & (1u << k)) continue;
      float w = 0.f, mag = 0.f, werr = 0.f;
      const float2* gp = reinterpret_cast<const float2*>(T.g2 + 2 * k * N);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const float g = __ldg(gp + i).x;
        w = fmaf(g, rf[i], w);
        mag = fmaf(fabsf(g), fabsf(rf[i]), mag);
        werr = fmaf(fabsf(g), e[i], werr);
      }
      if (!(fmaf(0x1p-19f, mag, w + werr) < tol)) ok = false;
      if (fmaf(-0x1p-19f, mag, w - werr) > tol) add |= 1u << k;  // provably violating
    }
  }
  if (!ok) {  // compaction into the fix or the repair queue
    if (fix_count && pos_ok && add) {
      a.ws_add[ch] = uint16_t(add);
      enqueue(fix_count, a.ws_fixq, int(ch));
    } else {
      enqueue(qcount, a.ws_queue, int(ch));
    }
    return;
  }
  // chi2 = ||r||^2 / pederr^2, the sum in double-float
  float ch2 = 0.f, cl2 = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    float p, q;
    two_prod(rh[i], rh[i], p, q);
    q = fmaf(2.f * rh[i], rl[i], q);
    df_acc(ch2, cl2, p, q);
  }
  // chi2 / pederr^2 in double-float: q1 = c / s2 rounded, then the remainder
  // c - q1 s2 (exact leading difference) divided once more (~2^-46 relative)
  double chi2;
  if (!bad) {
    const float q1 = __fdiv_rn(ch2, s2h);
    float p, q;
    two_prod(q1, s2h, p, q);
    const float rem = __fadd_rn(__fsub_rn(ch2, p), __fsub_rn(cl2, fmaf(q1, s2l, q)));
    chi2 = double(q1) + double(__fdiv_rn(rem, s2h));
  } else {
    chi2 = (double(ch2) + double(cl2)) / (sig * sig);
  }
  for (int k = K; k < a.amp_stride && k < KMAX; ++k) out[k] = 0.;
  a.chi2[ch] = chi2;
  if (a.intime) a.intime[ch] = T.intime_col >= 0 ? xin : 0.;
  if (a.active_mask) a.active_mask[ch] = support;
  if (a.status) {
    uint8_t st = 0;
    if (!(finite && finite64(chi2))) st |= CH_NONFINITE;
    if (bad) st |= CH_BADINPUT;
    a.status[ch] = st;
  }
  if (a.iters) {
    const int adds = int(cnt & 255u), solves = int(cnt >> 8) + 1;
    a.iters[ch] = 1 | ((adds < 4095 ? adds : 4095) << 8) | ((solves < 4095 ? solves : 4095) << 20);
  }
  if (a.flops) a.flops[ch] = double(K + 4);
}

}  // namespace
}  // namespace mfgb
