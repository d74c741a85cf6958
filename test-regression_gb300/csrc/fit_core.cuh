// The per-channel multifit of PulseChiSqSNNLS::DoFit
// (multifit_cpu/src/PulseChiSqSNNLS.cpp:21-273) as device routines over a
// scalar type T: the linalgebra primitives (linalgebra/interface/
// cholesky.hpp:8-38, substitution.hpp:10-50, fused_cholesky_substitution.hpp:
// 18-102), the in-place FNNLS with the incremental Cholesky
// (nnls/src/inplace_fnnls.cu:72-233, nnls/src/inplace_fnnls_test_cholesky.cu:
// 35-227), updateCov, ComputeChiSq, Minimize and ComputeApproxUncertainty.
//
// With T = double this is the plain FP64 drop-in (fit_fp64.cu, compiled
// --fmad=false: every accumulation is an explicit fused multiply-add with the
// index ascending, each triangular solve divides once by the diagonal, so the
// kernel reproduces the CPU oracle bit for bit).
//
// Per-thread storage. A thread's working set lives in local memory, cached
// by L1 and L2; with ~400 resident threads per SM a 5 KB set overflowed both
// and every access went to DRAM. So it is kept small: triangular factors and
// the symmetric normal matrix are stored packed (row i of the lower triangle
// at tri(i) = i(i+1)/2, 55 values for K = 10 instead of 100), the covariance
// is factored in place, the pulse matrix is read from the condition set (the
// kernel's parameters) instead of a per-thread copy, and the FNNLS factor
// reuses the whitened matrix's buffer once the normal equations are formed.
// Only where values are stored changes; every operation and its order stay.
#pragma once
#include <cfloat>

#include "mf_internal.h"

namespace mfgb {
namespace {

template <typename T>
struct Big;
template <>
struct Big<double> {
  static constexpr double value = DBL_MAX;
};

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ double sqrtT(double a) { return sqrt(a); }
__device__ __forceinline__ double fabsT(double a) { return fabs(a); }

constexpr int KTRI = KMAX * (KMAX + 1) / 2;

// start of row i of a packed lower triangle
__device__ __forceinline__ int tri(int i) { return i * (i + 1) / 2; }

// element (i, j) of a symmetric matrix stored as its packed lower triangle
template <typename T>
__device__ __forceinline__ T& sym(T* M, int i, int j) {
  return i >= j ? M[tri(i) + j] : M[tri(j) + i];
}

struct Flop {
  double v;
  __device__ __forceinline__ void fma(double k) { v += 2 * k; }
  __device__ __forceinline__ void op(double k) { v += k; }
};

template <bool COUNT>
struct Counter {
  Flop f{0};
  __device__ __forceinline__ void fma(double k) {
    if (COUNT) f.fma(k);
  }
  __device__ __forceinline__ void op(double k) {
    if (COUNT) f.op(k);
  }
};

// linalgebra/interface/cholesky.hpp:8-38, in place: L holds the packed lower
// triangle of the matrix on entry and its factor on return (element (i, j) is
// read once, just before the factor's (i, j) is written over it).
// R: also keep the reciprocals of the diagonal in rinv and multiply by them
// instead of dividing (one division per row: the per-channel form's FP64
// continuation, which needs no bit parity with the oracle)
template <bool C, typename T, bool R = false>
__device__ __forceinline__ void chol_rows(T* L, int n, Counter<C>& f, T* rinv = nullptr) {
  for (int i = 0; i < n; ++i) {
    T sumsq = 0;
    for (int j = 0; j < i; ++j) {
      T s2 = 0;
      for (int k = 0; k < j; ++k) s2 = fmaT(L[tri(i) + k], L[tri(j) + k], s2);
      const T v = R ? (L[tri(i) + j] - s2) * rinv[j] : (L[tri(i) + j] - s2) / L[tri(j) + j];
      L[tri(i) + j] = v;
      sumsq = fmaT(v, v, sumsq);
      f.fma(j + 1);
      f.op(2);
    }
    L[tri(i) + i] = sqrtT(L[tri(i) + i] - sumsq);
    if (R) rinv[i] = T(1) / L[tri(i) + i];
    f.op(2);
  }
}

// linalgebra/interface/substitution.hpp:10-26 (L packed; b(i) gives the
// right-hand side's element i)
template <bool C, typename T, bool R = false, typename Rhs>
__device__ __forceinline__ void fwd(const T* L, Rhs&& b, T* y, int n, Counter<C>& f, const T* rinv = nullptr) {
  for (int i = 0; i < n; ++i) {
    T t = b(i);
    for (int j = 0; j < i; ++j) t = fmaT(-L[tri(i) + j], y[j], t);
    y[i] = R ? t * rinv[i] : t / L[tri(i) + i];
    f.fma(i);
    f.op(1);
  }
}

// linalgebra/interface/substitution.hpp:34-50 (L^T x = y, L packed)
template <bool C, typename T>
__device__ __forceinline__ void bwd(const T* L, const T* y, T* x, int n, Counter<C>& f) {
  for (int i = n - 1; i >= 0; --i) {
    T t = y[i];
    for (int j = i + 1; j < n; ++j) t = fmaT(-L[tri(j) + i], x[j], t);
    x[i] = t / L[tri(i) + i];
    f.fma(n - 1 - i);
    f.op(1);
  }
}

// linalgebra/interface/fused_cholesky_substitution.hpp:18-59 (M symmetric,
// M and L packed lower triangles)
template <bool C, typename T>
__device__ __forceinline__ void rc_add(const T* M, T* L, const T* b, T* y, int view, Counter<C>& f) {
  const int row = view - 1;
  T sum = 0, total = b[row];
  for (int col = 0; col < row; ++col) {
    T s2 = 0;
    for (int j = 0; j < col; ++j) s2 = fmaT(L[tri(row) + j], L[tri(col) + j], s2);
    const T v = (M[tri(row) + col] - s2) / L[tri(col) + col];
    total = fmaT(-v, y[col], total);
    sum = fmaT(v, v, sum);
    L[tri(row) + col] = v;
    f.fma(col + 3);
    f.op(2);
  }
  const T d = sqrtT(M[tri(row) + row] - sum);
  L[tri(row) + row] = d;
  y[row] = total / d;
  f.op(3);
}

// linalgebra/interface/fused_cholesky_substitution.hpp:64-102 (M symmetric,
// M and L packed lower triangles)
template <bool C, typename T>
__device__ __forceinline__ void inbetween_removal(const T* M, T* L, const T* b, T* y, int pos, int view,
                                                  Counter<C>& f) {
  for (int i = pos; i < view; ++i) {
    T sumsq = 0, total = b[i];
    for (int j = 0; j < i; ++j) {
      T s2 = 0;
      for (int k = 0; k < j; ++k) s2 = fmaT(L[tri(i) + k], L[tri(j) + k], s2);
      const T v = (M[tri(i) + j] - s2) / L[tri(j) + j];
      L[tri(i) + j] = v;
      total = fmaT(-v, y[j], total);
      sumsq = fmaT(v, v, sumsq);
      f.fma(j + 2);
      f.op(2);
    }
    const T d = sqrtT(M[tri(i) + i] - sumsq);
    L[tri(i) + i] = d;
    y[i] = total / d;
    f.op(3);
  }
}

template <typename T>
__device__ __forceinline__ void swap_d(T& a, T& b) {
  const T t = a;
  a = b;
  b = t;
}

// symmetric permutation of indices a and b of an n x n symmetric matrix
// stored as its packed lower triangle: (a, a) <-> (b, b) and (a, k) <-> (b, k)
// for every other k; (a, b) stays
template <typename T>
__device__ __forceinline__ void swap_sym(T* M, int n, int a, int b) {
  if (a == b) return;
  swap_d(M[tri(a) + a], M[tri(b) + b]);
  for (int k = 0; k < n; ++k)
    if (k != a && k != b) swap_d(sym(M, a, k), sym(M, b, k));
}

struct FnnlsOut {
  int outer, inner, converged;
  uint16_t mask;
};

// FNNLS, nnls/src/inplace_fnnls.cu:72-233 with the incremental factor.
// A: N x K column-major (at least KTRI values: once the normal equations are
// formed the buffer holds the packed factor of the passive block), b: N,
// x: K warm start in / solution out.
// start 0: the reference's start (empty passive set, warm x);
// start 1: passive set seeded with the support of the warm x (ascending).
template <int NT, int KT, bool C, typename T>
__device__ void fnnls(T* A, const T* b, T* x, int N, int K, T eps, int max_iter, int start, FnnlsOut& o,
                      Counter<C>& f) {
  if (NT > 0) N = NT;
  if (KT > 0) K = KT;
  T AtA[KTRI], Atb[KMAX], s[KMAX], y[KMAX];
  int8_t perm[KMAX];
  for (int i = 0; i < K; ++i) {
    for (int j = i; j < K; ++j) {
      T acc = 0;
      for (int k = 0; k < N; ++k) acc = fmaT(A[i * N + k], A[j * N + k], acc);
      AtA[tri(j) + i] = acc;
      f.fma(N);
    }
  }
  for (int i = 0; i < K; ++i) {
    T acc = 0;
    for (int k = 0; k < N; ++k) acc = fmaT(A[i * N + k], b[k], acc);
    Atb[i] = acc;
    f.fma(N);
  }
  T* const L = A;  // A is not read again
  for (int i = 0; i < K; ++i) perm[i] = int8_t(i);

  int nP = 0, outer = 0, inner = 0, converged = 0;

  auto swap_in = [&](int p, int q) {
    swap_sym(AtA, K, p, q);
    swap_d(Atb[p], Atb[q]);
    swap_d(x[p], x[q]);
    const int8_t t = perm[p];
    perm[p] = perm[q];
    perm[q] = t;
  };

  // inner loop; `added` rows were just appended to the passive block
  auto inner_loop = [&](int added) {
    int inner_iteration = 0, position_removed = -1;
    while (nP > 0) {
      ++inner;
      if (nP == 1) {
        const T l00 = sqrtT(AtA[0]);
        L[0] = l00;
        y[0] = Atb[0] / l00;
        position_removed = -1;
        f.op(2);
      } else if (inner_iteration == 0) {
        for (int r = nP - added + 1; r <= nP; ++r) {
          if (r == 1) {
            const T l00 = sqrtT(AtA[0]);
            L[0] = l00;
            y[0] = Atb[0] / l00;
            f.op(2);
          } else {
            rc_add(AtA, L, Atb, y, r, f);
          }
        }
      } else {
        inbetween_removal(AtA, L, Atb, y, position_removed, nP, f);
      }
      bwd(L, y, s, nP, f);

      T smin = s[0];
      for (int i = 1; i < nP; ++i) smin = (s[i] < smin) ? s[i] : smin;
      if (smin > T(0)) {
        for (int i = 0; i < nP; ++i) x[i] = s[i];
        break;
      }
      T alpha = Big<T>::value;
      int alpha_idx = 0;
      for (int i = 0; i < nP; ++i) {
        if (s[i] <= T(0)) {
          const T ratio = x[i] / (x[i] - s[i]);
          f.op(2);
          if (ratio < alpha) {
            alpha = ratio;
            alpha_idx = i;
          }
        }
      }
      if (alpha == Big<T>::value) {
        for (int i = 0; i < nP; ++i) x[i] = s[i];
        break;
      }
      for (int i = 0; i < nP; ++i) x[i] = fmaT(alpha, s[i] - x[i], x[i]);
      f.fma(nP);
      f.op(nP);
      x[alpha_idx] = 0;
      --nP;
      swap_in(nP, alpha_idx);
      position_removed = alpha_idx;
      ++inner_iteration;
    }
  };

  if (start == 1) {
    // columns with x_k > 0 and a non-zero whitened norm (the MINOS refits
    // zero the in-time column and hold its amplitude fixed)
    for (int k = 0; k < K; ++k)
      if (x[k] > T(0) && AtA[tri(k) + k] > T(0)) swap_in(nP++, k);
    if (nP > 0) inner_loop(nP);
  }

  for (int iter = 0; iter < max_iter; ++iter) {
    if (nP == K) {
      converged = 1;
      break;
    }
    int imax = nP;
    T wmax = 0;
    for (int i = nP; i < K; ++i) {
      T acc = 0;
      for (int j = 0; j < K; ++j) acc = fmaT(sym(AtA, i, j), x[j], acc);
      const T w = Atb[i] - acc;
      f.fma(K);
      f.op(1);
      if (i == nP || w > wmax) {
        wmax = w;
        imax = i;
      }
    }
    if (wmax < eps) {
      converged = 1;
      break;
    }
    ++outer;
    swap_in(nP, imax);
    ++nP;
    inner_loop(1);
  }
  T* const xo = s;  // s is not read again
  for (int i = 0; i < K; ++i) xo[perm[i]] = x[i];
  uint16_t mask = 0;
  for (int i = 0; i < nP; ++i) mask |= uint16_t(1u << perm[i]);
  for (int i = 0; i < K; ++i) x[i] = xo[i];
  o.outer += outer;
  o.inner += inner;
  o.converged = converged;
  o.mask = mask;
}

// Per-channel state of PulseChiSqSNNLS (multifit_cpu/interface/PulseChiSqSNNLS.h:44-58).
template <typename T>
struct FitState {
  T samp[KMAX];
  T amp[KMAX];
  T LC[KTRI];        // lower factor of the covariance, packed rows
  T LCr[KMAX];       // reciprocals of LC's diagonal (kept by the reciprocal variant only)
  int zcol;          // pulse-matrix column held at zero (the error refits' in-time column), or -1
  T chisq;
  FnnlsOut st;
  int outer_iters;
  int outer_maxed;
};

// element (i, k) of the pulse matrix the fit uses: the condition set's, with
// column S.zcol at zero
template <typename T>
__device__ __forceinline__ T pulse(const DevConditions& c, const FitState<T>& S, int N, int k, int i) {
  return k == S.zcol ? T(0) : T(c.P[k * N + i]);
}

// updateCov, multifit_cpu/src/PulseChiSqSNNLS.cpp:169-194
// (the covariance is formed in S.LC and factored there)
template <int NT, int KT, bool C, typename T, bool R = false>
__device__ void update_cov(const DevConditions& c, int N, int K, T pederr, FitState<T>& S, Counter<C>& f) {
  T* const M = S.LC;
  const T ped2 = pederr * pederr;
  f.op(1);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j) M[tri(i) + j] = ped2 * T(c.R[j * N + i]);
  f.op(N * (N + 1) / 2);
  if (c.has_fpc) {
    const int NF = N + 9;
    for (int k = 0; k < K; ++k) {
      if (S.amp[k] == T(0)) continue;
      const int bx = c.bxs[k];
      const int first = bx + 3 > 0 ? bx + 3 : 0;
      const int offset = 7 - 3 - bx;
      const T ampsq = S.amp[k] * S.amp[k];
      const int ns = N - first;
      for (int a = 0; a < ns; ++a)
        for (int cc = 0; cc <= a; ++cc) {
          const int i = first + a, j = first + cc;
          M[tri(i) + j] = fmaT(ampsq, T(c.fpc[(j + offset) * NF + (i + offset)]), M[tri(i) + j]);
        }
      f.op(1);
      f.fma(ns * (ns + 1) / 2);
    }
  }
  chol_rows<C, T, R>(S.LC, N, f, S.LCr);
}

// ComputeChiSq, multifit_cpu/src/PulseChiSqSNNLS.cpp:196-200
template <bool C, typename T, bool R = false>
__device__ T compute_chisq(const DevConditions& c, int N, int K, const FitState<T>& S, Counter<C>& f) {
  T r[KMAX], z[KMAX];
  for (int i = 0; i < N; ++i) {
    T acc = 0;
    for (int k = 0; k < K; ++k) acc = fmaT(pulse(c, S, N, k, i), S.amp[k], acc);
    r[i] = acc - S.samp[i];
  }
  f.fma(N * K);
  f.op(N);
  fwd<C, T, R>(S.LC, [&](int i) { return r[i]; }, z, N, f, S.LCr);
  T chi2 = 0;
  for (int i = 0; i < N; ++i) chi2 = fmaT(z[i], z[i], chi2);
  f.fma(N);
  return chi2;
}

// One outer iteration of Minimize (multifit_cpu/src/PulseChiSqSNNLS.cpp:
// 149-166, with NNLS :219-273): covariance and its factor, whitening, FNNLS
// from the current amplitudes, chi2; returns |delta chi2| < tol. `act` = the
// lanes of the warp running an iteration together: they reconverge after the
// divergent FNNLS, because on this GPU an FP64 warp instruction costs the full
// pipe time whatever the number of active lanes, so chi2 must be issued once
// for all of them rather than once per group of lanes that left FNNLS together.
template <int NT, int KT, bool C, typename T, bool R = false>
__device__ bool outer_iteration(const DevConditions& c, const DevOptions& o, int N, int K, T pederr,
                                FitState<T>& S, Counter<C>& f, unsigned act) {
  update_cov<NT, KT, C, T, R>(c, N, K, pederr, S, f);
  T A[KMAX * KMAX], b[KMAX];
  for (int k = 0; k < K; ++k) fwd<C, T, R>(S.LC, [&](int i) { return pulse(c, S, N, k, i); }, A + k * N, N, f, S.LCr);
  fwd<C, T, R>(S.LC, [&](int i) { return S.samp[i]; }, b, N, f, S.LCr);
  fnnls<NT, KT>(A, b, S.amp, N, K, T(o.nnls_eps), o.max_iter_nnls, o.nnls_start, S.st, f);
  __syncwarp(act);
  const T now = compute_chisq<C, T, R>(c, N, K, S, f);
  const T delta = now - S.chisq;
  f.op(1);
  S.chisq = now;
  ++S.outer_iters;
  return fabsT(delta) < T(o.dchi2_tol);
}

// ComputeApproxUncertainty, multifit_cpu/src/PulseChiSqSNNLS.cpp:202-207
template <bool C, typename T, bool R = false>
__device__ T approx_uncertainty(const DevConditions& c, int N, const FitState<T>& S, int k, Counter<C>& f) {
  T z[KMAX];
  fwd<C, T, R>(S.LC, [&](int i) { return pulse(c, S, N, k, i); }, z, N, f, S.LCr);
  T n2 = 0;
  for (int i = 0; i < N; ++i) n2 = fmaT(z[i], z[i], n2);
  f.fma(N);
  f.op(2);
  return T(1) / sqrtT(n2);
}
// Coalesced staging of a warp's channel rows through shared memory: rows
// [ch0, ch0 + nw) (nw <= 32) of a row-major array with `stride` elements per
// row, `width` <= KMAX elements of each, into `rows` (KMAX per row). Lane
// `lane` moves elements lane, lane + 32, ... of the warp's nw x width block,
// so consecutive lanes read consecutive addresses (a channel's own row, read
// by its thread, is 80 bytes wide: 32 lanes reading their own rows touch 32
// rows per instruction).
__device__ __forceinline__ void stage_rows_in(const double* src, int64_t stride, int64_t ch0, int nw, int width,
                                              double* rows, int lane) {
  for (int e = lane; e < nw * width; e += 32) {
    const int r = e / width, i = e - r * width;
    rows[r * KMAX + i] = src[(ch0 + r) * stride + i];
  }
}

// DoFit (multifit_cpu/src/PulseChiSqSNNLS.cpp:21-147) of one channel as a
// sequence of steps, so that a lane can take its next channel as soon as its
// own is done instead of idling until the slowest lane of its warp finishes
// (channels need 2 or 3 outer iterations, and the error estimate one or two
// more Minimize calls). The per-channel arithmetic and its order are those
// of DoFit; only the schedule across channels changes.
//
// start() loads the channel. prepare() moves on while the current Minimize
// has stopped (main fit -> refit with the in-time amplitude held above its
// value -> refit held below it -> done) and returns true when an outer
// iteration is to run, false once the channel is finished and its outputs
// are written. iterate() runs that outer iteration.
//
// With a.seeded the main Minimize's first outer iteration has been done
// already and its amplitudes, chi2 and status are read from the outputs; the
// loop goes on from the second iteration, with the reference's stopping rule
// against that chi2 (against 0 after the first iteration). seeded = 1: the
// per-channel form of the mixed and FP32 precisions (with the amplitudes at
// zero the covariance is pederr^2 samplecor, the problem of the passive-set
// tables); seeded = 2: the FP64 kernel's own first pass, whose FNNLS
// counters (iters) and executed flops are carried on too, so that the two
// passes together give the single fit's outputs bit for bit.
template <int NT, int KT, bool C, bool R = false>
struct ChannelFit {
  FitState<double> S;
  double samp0[KMAX];   // the channel's samples (the refits fit shifted copies)
  double ampmin[KMAX];  // the main fit's amplitudes
  double pederr, chisq0, x0, approxerr, sigmaplus, err;
  int64_t ch;
  FnnlsOut main_st;
  int main_outer, main_maxed;
  int it;     // outer iteration of the current Minimize
  int phase;  // 0 main fit, 1 upper refit, 2 lower refit
  bool done, bad;
  Counter<C> f;

  // samples: the channel's N samples (a warp's staging row)
  __device__ void start(const FitArgs& a, const DevConditions& c, int64_t channel, const double* samples) {
    const int N = NT > 0 ? NT : c.N;
    const int K = KT > 0 ? KT : c.K;
    ch = channel;
    f = Counter<C>{};
    pederr = a.pederr[ch];
    bad = !isfinite(pederr);
    for (int i = 0; i < N; ++i) {
      samp0[i] = samples[i];
      S.samp[i] = samples[i];
      bad = bad || !isfinite(samples[i]);
    }
    S.zcol = -1;
    for (int k = 0; k < K; ++k) S.amp[k] = 0.;
    S.chisq = 0.;
    S.st = FnnlsOut{0, 0, 0, 0};
    S.outer_iters = 0;
    S.outer_maxed = 0;
    it = 0;
    done = false;
    phase = 0;
    err = 0.;
    if (a.seeded) {
      const double* seed = a.amplitudes + ch * a.amp_stride;
      const bool maxed = a.status && (a.status[ch] & CH_NNLS_MAXITER);
      if (a.opt.compute_errors && fabs(a.chi2[ch]) < a.opt.dchi2_tol) {
        // the loop stops at once: the error refits need the first iteration's
        // covariance factor, that of pederr^2 samplecor
        update_cov<NT, KT, C, double, R>(c, N, K, pederr, S, f);
      }
      for (int k = 0; k < K; ++k) S.amp[k] = seed[k];
      S.chisq = a.chi2[ch];
      S.st.converged = maxed ? 0 : 1;
      S.outer_iters = 1;
      if (a.seeded == 2) {
        if (a.iters) {
          S.st.outer = (a.iters[ch] >> 8) & 0xfff;
          S.st.inner = (a.iters[ch] >> 20) & 0xfff;
        }
        if (C && a.flops) f.f.v = a.flops[ch];
      }
      it = 1;
      done = fabs(S.chisq) < a.opt.dchi2_tol;
    }
  }

  __device__ bool prepare(const FitArgs& a, const DevConditions& c) {
    const int N = NT > 0 ? NT : c.N;
    const int K = KT > 0 ? KT : c.K;
    for (;;) {
      if (!done && it < a.opt.max_iter_outer) return true;
      // the current Minimize has stopped
      if (!done) S.outer_maxed = 1;
      const int kin = c.intime_col;
      if (phase == 0) {
        main_st = S.st;
        main_outer = S.outer_iters;
        main_maxed = S.outer_maxed;
        for (int k = 0; k < K; ++k) ampmin[k] = S.amp[k];
        if (!(a.opt.compute_errors && kin >= 0)) break;
        approxerr = approx_uncertainty<C, double, R>(c, N, S, kin, f);
        chisq0 = S.chisq;
        x0 = ampmin[kin];
        S.zcol = kin;  // the in-time column held fixed
        const double xplus = x0 + approxerr;
        S.amp[kin] = xplus;
        for (int i = 0; i < N; ++i) S.samp[i] = fma(-xplus, c.P[kin * N + i], samp0[i]);
        phase = 1;
      } else if (phase == 1) {
        const double xplus = x0 + approxerr;
        const double chip = compute_chisq<C, double, R>(c, N, K, S, f);
        sigmaplus = fabs(xplus - x0) / sqrt(chip - chisq0);
        if (!(x0 / sigmaplus > 0.5)) {
          err = sigmaplus;
          S.chisq = chisq0;
          break;
        }
        const double xminus = (x0 - approxerr) > 0. ? (x0 - approxerr) : 0.;
        S.amp[kin] = xminus;
        for (int i = 0; i < N; ++i) S.samp[i] = fma(-xminus, c.P[kin * N + i], samp0[i]);
        phase = 2;
      } else {
        const double xminus = (x0 - approxerr) > 0. ? (x0 - approxerr) : 0.;
        const double chim = compute_chisq<C, double, R>(c, N, K, S, f);
        const double sigmaminus = fabs(xminus - x0) / sqrt(chim - chisq0);
        err = 0.5 * (sigmaplus + sigmaminus);
        S.chisq = chisq0;
        break;
      }
      // a refit: the whole Minimize loop, from the chi2 of the main fit
      it = 0;
      done = false;
    }
    finish(a, c);
    return false;
  }

  __device__ void iterate(const FitArgs& a, const DevConditions& c, unsigned act) {
    const int N = NT > 0 ? NT : c.N;
    const int K = KT > 0 ? KT : c.K;
    done = outer_iteration<NT, KT, C, double, R>(c, a.opt, N, K, pederr, S, f, act);
    ++it;
  }

  __device__ void finish(const FitArgs& a, const DevConditions& c) {
    const int K = KT > 0 ? KT : c.K;
    double* out = a.amplitudes + ch * a.amp_stride;
    bool finite = isfinite(S.chisq);
    for (int k = 0; k < K; ++k) {
      out[k] = ampmin[k];
      finite = finite && isfinite(ampmin[k]);
    }
    for (int k = K; k < a.amp_stride && k < KMAX; ++k) out[k] = 0.;
    a.chi2[ch] = S.chisq;
    if (a.intime) a.intime[ch] = c.intime_col >= 0 ? ampmin[c.intime_col] : 0.;
    if (a.errors) a.errors[ch] = err;
    if (a.active_mask) {
      // support of X(): the last FNNLS call restarts from an empty passive set
      // and usually stops at once, so its passive set is not the fitted set
      uint16_t support = 0;
      for (int k = 0; k < K; ++k)
        if (ampmin[k] > 0.) support |= uint16_t(1u << k);
      a.active_mask[ch] = support;
    }
    if (a.status) {
      uint8_t st = 0;
      if (!main_st.converged) st |= CH_NNLS_MAXITER;
      if (main_maxed) st |= CH_OUTER_MAXITER;
      if (!finite) st |= CH_NONFINITE;
      if (bad) st |= CH_BADINPUT;
      a.status[ch] = st;
    }
    if (a.iters) {
      const int o8 = main_outer < 255 ? main_outer : 255;
      const int fo = main_st.outer < 4095 ? main_st.outer : 4095;
      const int fi = main_st.inner < 4095 ? main_st.inner : 4095;
      a.iters[ch] = o8 | (fo << 8) | (fi << 20);
    }
    if (C && a.flops) a.flops[ch] = f.f.v;
  }
};

}  // namespace
}  // namespace mfgb
