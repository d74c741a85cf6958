// CPU oracle for the multifit hot path. TEST INFRASTRUCTURE ONLY: the tests,
// the smoke check and the CPU-baseline leg of the benchmark call it as the
// checker. No product code links it.
//
// It restates, in plain C++17 FP64 without Eigen, the per-channel fit of the
// reference's multifit_cpu:
//   PulseChiSqSNNLS::DoFit            multifit_cpu/src/PulseChiSqSNNLS.cpp:21-147
//   PulseChiSqSNNLS::Minimize         multifit_cpu/src/PulseChiSqSNNLS.cpp:149-166
//   PulseChiSqSNNLS::updateCov        multifit_cpu/src/PulseChiSqSNNLS.cpp:169-194
//   PulseChiSqSNNLS::ComputeChiSq     multifit_cpu/src/PulseChiSqSNNLS.cpp:196-200
//   ComputeApproxUncertainty          multifit_cpu/src/PulseChiSqSNNLS.cpp:202-207
//   PulseChiSqSNNLS::NNLS             multifit_cpu/src/PulseChiSqSNNLS.cpp:219-273
//   inplace_fnnls                     nnls/src/inplace_fnnls.cu:72-233
//   inplace_fnnls_test_cholesky       nnls/src/inplace_fnnls_test_cholesky.cu:35-227
//   cholesky_decomp                   linalgebra/interface/cholesky.hpp:8-38
//   solve_forward/backward_substitution linalgebra/interface/substitution.hpp:10-50
//   fused ..._rcaddition / _inbetween_removal
//                                     linalgebra/interface/fused_cholesky_substitution.hpp:18-102
//   swap_row_column                   linalgebra/interface/common.hpp:11-42
//
// Canonical operation order. Eigen (a third-party dependency the reference
// does not vendor, version unpinned) fixes no portable rounding order for its
// vectorised reductions, so bit parity with an Eigen build cannot be pinned.
// This oracle fixes one order and the GPU FP64 kernel follows the same one:
//   * every accumulation "acc +/-= a*b" is one fused multiply-add, summed with
//     the index ascending from an exact zero (or from the minuend);
//   * the Cholesky factor is formed element by element with the formulas of
//     the reference's hand-written linalgebra headers (off-diagonal:
//     (M_ij - sum_k L_ik L_jk) / L_jj; diagonal: sqrt(M_ii - sum_j L_ij^2));
//     the column-oriented LLT that inplace_fnnls calls computes the same
//     per-element formula, so one routine serves both;
//   * triangular solves are sequential subtractions t -= L_ij * y_j followed
//     by one IEEE division by the diagonal, as in substitution.hpp;
//   * division and sqrt are IEEE-754 correctly rounded.
// With this order the "fresh LLT per inner step" FNNLS of inplace_fnnls and
// the incremental add/remove FNNLS of inplace_fnnls_test_cholesky produce the
// same bits: an incremental row is computed by exactly the formulas a fresh
// factorisation uses for that row, and rows above the change are untouched.
//
// Build: oracle/build_oracle.py (g++ -O3 -ffp-contract=off, so that only the
// explicit std::fma calls fuse).

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr int KMAX = 10;  // maximum samples (N) and pulses (K) per channel

// Counters of executed floating-point work, used for the roofline figure:
// fma counts 2 flops, add/sub/mul/div/sqrt 1 each.
struct Flops {
  double v = 0;
  inline void fma(double k = 1) { v += 2 * k; }
  inline void op(double k = 1) { v += k; }
};

// Every a*b + c of the canonical order is one fused multiply-add. Built with
// ORACLE_SEPARATE_ROUNDING, the same expressions round the product and the sum
// separately (the file is compiled -ffp-contract=off): that build is the one
// compared bit for bit with the reference's plain-C FNNLS compiled likewise.
#ifdef ORACLE_SEPARATE_ROUNDING
inline double FMA(double a, double b, double c) { return a * b + c; }
#else
inline double FMA(double a, double b, double c) { return std::fma(a, b, c); }
#endif

// ---------------------------------------------------------------------------
// linalgebra restatement (row-major square storage of leading dimension ld)
// ---------------------------------------------------------------------------

// linalgebra/interface/cholesky.hpp:8-38
void cholesky_rows(const double* M, double* L, int ld, int row_begin, int row_end, Flops* f) {
  for (int i = row_begin; i < row_end; ++i) {
    double sumsq = 0;
    for (int j = 0; j < i; ++j) {
      double s2 = 0;
      for (int k = 0; k < j; ++k) s2 = FMA(L[i * ld + k], L[j * ld + k], s2);
      const double v = (M[i * ld + j] - s2) / L[j * ld + j];
      L[i * ld + j] = v;
      sumsq = FMA(v, v, sumsq);
      if (f) { f->fma(j + 1); f->op(2); }
    }
    L[i * ld + i] = std::sqrt(M[i * ld + i] - sumsq);
    if (f) f->op(2);
  }
}

// linalgebra/interface/substitution.hpp:10-26 (forward, lower L)
void forward_subst(const double* L, int ld, const double* b, double* y, int n, Flops* f) {
  for (int i = 0; i < n; ++i) {
    double t = b[i];
    for (int j = 0; j < i; ++j) t = FMA(-L[i * ld + j], y[j], t);
    y[i] = t / L[i * ld + i];
    if (f) { f->fma(i); f->op(1); }
  }
}

// linalgebra/interface/substitution.hpp:34-50 (solves L^T x = y with lower L)
void backward_subst(const double* L, int ld, const double* y, double* x, int n, Flops* f) {
  for (int i = n - 1; i >= 0; --i) {
    double t = y[i];
    for (int j = i + 1; j < n; ++j) t = FMA(-L[j * ld + i], x[j], t);
    x[i] = t / L[i * ld + i];
    if (f) { f->fma(n - 1 - i); f->op(1); }
  }
}

// linalgebra/interface/fused_cholesky_substitution.hpp:18-59. M, b and y are
// in the same (permuted) frame; rows [0, view-1) of L and y are valid on entry.
void fused_rc_addition(const double* M, double* L, int ld, const double* b, double* y, int view, Flops* f) {
  const int row = view - 1;
  double sum = 0;
  double total = b[row];
  for (int col = 0; col < row; ++col) {
    double s2 = 0;
    for (int j = 0; j < col; ++j) s2 = FMA(L[row * ld + j], L[col * ld + j], s2);
    const double v = (M[row * ld + col] - s2) / L[col * ld + col];
    total = FMA(-v, y[col], total);
    sum = FMA(v, v, sum);
    L[row * ld + col] = v;
    if (f) { f->fma(col + 3); f->op(2); }
  }
  const double d = std::sqrt(M[row * ld + row] - sum);
  L[row * ld + row] = d;
  y[row] = total / d;
  if (f) f->op(3);
}

// linalgebra/interface/fused_cholesky_substitution.hpp:64-102
void fused_inbetween_removal(const double* M, double* L, int ld, const double* b, double* y, int position,
                             int view, Flops* f) {
  for (int i = position; i < view; ++i) {
    double sumsq = 0;
    double total = b[i];
    for (int j = 0; j < i; ++j) {
      double s2 = 0;
      for (int k = 0; k < j; ++k) s2 = FMA(L[i * ld + k], L[j * ld + k], s2);
      const double v = (M[i * ld + j] - s2) / L[j * ld + j];
      L[i * ld + j] = v;
      total = FMA(-v, y[j], total);
      sumsq = FMA(v, v, sumsq);
      if (f) { f->fma(j + 2); f->op(2); }
    }
    const double d = std::sqrt(M[i * ld + i] - sumsq);
    L[i * ld + i] = d;
    y[i] = total / d;
    if (f) f->op(3);
  }
}

// Symmetric row+column exchange of a full square matrix (Eigen's
// AtA.col(a).swap(AtA.col(b)); AtA.row(a).swap(AtA.row(b)) in
// nnls/src/inplace_fnnls.cu:157-158).
void swap_sym(double* M, int ld, int n, int a, int b) {
  if (a == b) return;
  for (int k = 0; k < n; ++k) std::swap(M[k * ld + a], M[k * ld + b]);
  for (int k = 0; k < n; ++k) std::swap(M[a * ld + k], M[b * ld + k]);
}

// ---------------------------------------------------------------------------
// FNNLS (nnls/src/inplace_fnnls.cu:72-233 and the incremental twin)
// ---------------------------------------------------------------------------

struct FnnlsStats {
  int outer_iters = 0;    // additions to the passive set
  int inner_solves = 0;   // passive-set solves
  int converged = 0;      // stopped by max_w < eps or an empty active set
  int passive = 0;        // final passive-set size
  uint16_t mask = 0;      // final passive set, original column order
};

// A: N x K column-major (A[k*N + i] = A(i,k)); b: N; x: K in/out (warm start).
// variant 0 = fresh LLT of the passive block per inner step (inplace_fnnls),
// variant 1 = incremental add / in-between removal (inplace_fnnls_test_cholesky).
// start 0 = the reference's start: empty passive set, x = the warm amplitudes
//           (nnls/src/inplace_fnnls.cu:97 with x from PulseChiSqSNNLS.cpp:258);
// start 1 = support start: the passive set is first seeded with the support of
//           the warm x (columns with x_k > 0, ascending), made feasible by the
//           inner loop, then the reference loop runs. With x = 0 both starts
//           are the same; with a KKT point as warm start, start 1 stops at once.
void inplace_fnnls(const double* A, const double* b, double* x, int N, int K, double eps, int max_iter,
                   int variant, int start, FnnlsStats* st, Flops* f) {
  double AtA[KMAX * KMAX], Atb[KMAX], s[KMAX], w[KMAX];
  double L[KMAX * KMAX], y[KMAX];
  int perm[KMAX];
  const int ld = KMAX;

  // transpose_multiply, nnls/src/inplace_fnnls.cu:11-25: AtA(i,j) = sum_k A(k,i) A(k,j)
  for (int i = 0; i < K; ++i) {
    for (int j = i; j < K; ++j) {
      double acc = 0;
      for (int k = 0; k < N; ++k) acc = FMA(A[i * N + k], A[j * N + k], acc);
      AtA[j * ld + i] = acc;
      AtA[i * ld + j] = acc;
      if (f) f->fma(N);
    }
  }
  // Atb = A^T b, nnls/src/inplace_fnnls.cu:117
  for (int i = 0; i < K; ++i) {
    double acc = 0;
    for (int k = 0; k < N; ++k) acc = FMA(A[i * N + k], b[k], acc);
    Atb[i] = acc;
    if (f) f->fma(N);
  }
  for (int i = 0; i < K; ++i) perm[i] = i;
  std::memset(L, 0, sizeof(L));

  int nP = 0;
  int outer = 0, inner = 0, converged = 0;

  auto swap_in = [&](int a, int c) {
    swap_sym(AtA, ld, K, a, c);
    std::swap(Atb[a], Atb[c]);
    std::swap(x[a], x[c]);
    std::swap(perm[a], perm[c]);
  };

  // Inner loop (nnls/src/inplace_fnnls.cu:175-230; incremental factor as in
  // nnls/src/inplace_fnnls_test_cholesky.cu:144-224). `added` rows were just
  // appended to the passive block and still need their factor rows.
  auto inner_loop = [&](int added) {
    int inner_iteration = 0;
    int position_removed = -1;
    while (nP > 0) {
      ++inner;
      if (variant == 0) {
        cholesky_rows(AtA, L, ld, 0, nP, f);
        forward_subst(L, ld, Atb, y, nP, f);
        backward_subst(L, ld, y, s, nP, f);
      } else {
        if (nP == 1) {
          const double l00 = std::sqrt(AtA[0]);
          L[0] = l00;
          y[0] = Atb[0] / l00;
          position_removed = -1;
          if (f) f->op(2);
        } else if (inner_iteration == 0) {
          for (int r = nP - added + 1; r <= nP; ++r) {
            if (r == 1) {
              const double l00 = std::sqrt(AtA[0]);
              L[0] = l00;
              y[0] = Atb[0] / l00;
              if (f) f->op(2);
            } else {
              fused_rc_addition(AtA, L, ld, Atb, y, r, f);
            }
          }
        } else {
          fused_inbetween_removal(AtA, L, ld, Atb, y, position_removed, nP, f);
        }
        backward_subst(L, ld, y, s, nP, f);
      }
      double smin = s[0];
      for (int i = 1; i < nP; ++i) smin = std::min(smin, s[i]);
      if (smin > 0.) {
        for (int i = 0; i < nP; ++i) x[i] = s[i];
        break;
      }
      // nnls/src/inplace_fnnls.cu:188-200
      double alpha = std::numeric_limits<double>::max();
      int alpha_idx = 0;
      for (int i = 0; i < nP; ++i) {
        if (s[i] <= 0.) {
          const double ratio = x[i] / (x[i] - s[i]);
          if (f) f->op(2);
          if (ratio < alpha) { alpha = ratio; alpha_idx = i; }
        }
      }
      if (alpha == std::numeric_limits<double>::max()) {
        for (int i = 0; i < nP; ++i) x[i] = s[i];
        break;
      }
      // nnls/src/inplace_fnnls.cu:215-229
      for (int i = 0; i < nP; ++i) x[i] = FMA(alpha, s[i] - x[i], x[i]);
      if (f) { f->fma(nP); f->op(nP); }
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
      if (x[k] > 0. && AtA[k * ld + k] > 0.) swap_in(nP++, k);
    if (nP > 0) inner_loop(nP);
  }

  for (int iter = 0; iter < max_iter; ++iter) {
    const int nActive = K - nP;
    if (!nActive) { converged = 1; break; }
    // w.tail = Atb.tail - (AtA * x).tail   (nnls/src/inplace_fnnls.cu:137)
    for (int i = nP; i < K; ++i) {
      double acc = 0;
      for (int j = 0; j < K; ++j) acc = FMA(AtA[i * ld + j], x[j], acc);
      w[i] = Atb[i] - acc;
      if (f) { f->fma(K); f->op(1); }
    }
    // maxCoeff: first maximum wins (nnls/src/inplace_fnnls.cu:143-144)
    int imax = nP;
    double wmax = w[nP];
    for (int i = nP + 1; i < K; ++i)
      if (w[i] > wmax) { wmax = w[i]; imax = i; }
    if (wmax < eps) { converged = 1; break; }
    ++outer;
    // move the new index into slot nP (nnls/src/inplace_fnnls.cu:157-166)
    swap_in(nP, imax);
    ++nP;
    inner_loop(1);
  }
  // x = x^T * P^T: x_out[perm[i]] = x[i]   (nnls/src/inplace_fnnls.cu:232)
  double xo[KMAX];
  for (int i = 0; i < K; ++i) xo[perm[i]] = x[i];
  uint16_t mask = 0;
  for (int i = 0; i < nP; ++i) mask |= uint16_t(1u << perm[i]);
  std::memcpy(x, xo, sizeof(double) * K);
  if (st) {
    st->outer_iters += outer;
    st->inner_solves += inner;
    st->converged = converged;
    st->passive = nP;
    st->mask = mask;
  }
}

// ---------------------------------------------------------------------------
// Per-channel fit (multifit_cpu PulseChiSqSNNLS)
// ---------------------------------------------------------------------------

struct FitConfig {
  int N, K;
  const double* P;     // N x K column-major pulse matrix
  const double* R;     // N x N sample correlation (samplecor), lower triangle read
  const double* fpc;   // (N+9) x (N+9) column-major fullpulsecov, or nullptr
  const int8_t* bxs;   // K BX offsets (used for fullpulsecov blocks and the in-time column)
  double eps;
  int max_iter_nnls;
  int max_iter_outer;
  double dchi2_tol;
  int variant;
  int start;
  int compute_errors;
};

struct FitState {
  double samp[KMAX];     // _sampvec
  double amp[KMAX];      // _ampvec
  double P[KMAX * KMAX]; // _pulsemat (column-major N x K)
  double C[KMAX * KMAX]; // _invcov lower triangle, row-major ld=KMAX
  double L[KMAX * KMAX]; // _covdecomp.matrixL(), row-major ld=KMAX
  double chisq;
  FnnlsStats st;
  int outer_iters;
  int nonfinite;
  int outer_maxed;
};

// updateCov, multifit_cpu/src/PulseChiSqSNNLS.cpp:169-194
void update_cov(const FitConfig& cfg, double pederr, FitState& S, Flops* f) {
  const int N = cfg.N;
  const double ped2 = pederr * pederr;
  if (f) f->op(1);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j) S.C[i * KMAX + j] = ped2 * cfg.R[j * N + i];
  if (f) f->op(N * (N + 1) / 2);
  if (cfg.fpc) {
    const int NF = N + 9;
    for (int k = 0; k < cfg.K; ++k) {
      if (S.amp[k] == 0.) continue;
      const int bx = cfg.bxs[k];
      const int first = std::max(0, bx + 3);
      const int offset = 7 - 3 - bx;
      const double ampsq = S.amp[k] * S.amp[k];
      const int ns = N - first;
      for (int a = 0; a < ns; ++a)
        for (int c = 0; c <= a; ++c) {
          const int i = first + a, j = first + c;
          S.C[i * KMAX + j] = FMA(ampsq, cfg.fpc[(j + offset) * NF + (i + offset)], S.C[i * KMAX + j]);
        }
      if (f) { f->op(1); f->fma(ns * (ns + 1) / 2); }
    }
  }
  // _covdecomp.compute(_invcov)
  cholesky_rows(S.C, S.L, KMAX, 0, N, f);
}

// ComputeChiSq, multifit_cpu/src/PulseChiSqSNNLS.cpp:196-200: ||L^-1 (P a - s)||^2
double compute_chisq(const FitConfig& cfg, const FitState& S, Flops* f) {
  const int N = cfg.N, K = cfg.K;
  double r[KMAX], z[KMAX];
  for (int i = 0; i < N; ++i) {
    double acc = 0;
    for (int k = 0; k < K; ++k) acc = FMA(S.P[k * N + i], S.amp[k], acc);
    r[i] = acc - S.samp[i];
  }
  if (f) { f->fma(N * K); f->op(N); }
  forward_subst(S.L, KMAX, r, z, N, f);
  double c = 0;
  for (int i = 0; i < N; ++i) c = FMA(z[i], z[i], c);
  if (f) f->fma(N);
  return c;
}

// NNLS, multifit_cpu/src/PulseChiSqSNNLS.cpp:219-273
void nnls_step(const FitConfig& cfg, FitState& S, Flops* f) {
  const int N = cfg.N, K = cfg.K;
  double A[KMAX * KMAX], b[KMAX];
  // A = L^-1 P (column by column), b = L^-1 s
  for (int k = 0; k < K; ++k) forward_subst(S.L, KMAX, S.P + k * N, A + k * N, N, f);
  forward_subst(S.L, KMAX, S.samp, b, N, f);
  double x[KMAX];
  std::memcpy(x, S.amp, sizeof(double) * K);
  inplace_fnnls(A, b, x, N, K, cfg.eps, cfg.max_iter_nnls, cfg.variant, cfg.start, &S.st, f);
  std::memcpy(S.amp, x, sizeof(double) * K);
}

// Minimize, multifit_cpu/src/PulseChiSqSNNLS.cpp:149-166
void minimize(const FitConfig& cfg, double pederr, FitState& S, Flops* f) {
  for (int it = 0; it < cfg.max_iter_outer; ++it) {
    update_cov(cfg, pederr, S, f);
    nnls_step(cfg, S, f);
    const double now = compute_chisq(cfg, S, f);
    const double delta = now - S.chisq;
    if (f) f->op(1);
    S.chisq = now;
    ++S.outer_iters;
    if (std::fabs(delta) < cfg.dchi2_tol) return;
  }
  S.outer_maxed = 1;
}

// ComputeApproxUncertainty, multifit_cpu/src/PulseChiSqSNNLS.cpp:202-207
double approx_uncertainty(const FitConfig& cfg, const FitState& S, int k, Flops* f) {
  double z[KMAX];
  forward_subst(S.L, KMAX, S.P + k * cfg.N, z, cfg.N, f);
  double n2 = 0;
  for (int i = 0; i < cfg.N; ++i) n2 = FMA(z[i], z[i], n2);
  if (f) { f->fma(cfg.N); f->op(2); }
  return 1. / std::sqrt(n2);
}

struct FitResult {
  double amp[KMAX];
  double chisq;
  double err;       // MINOS-like in-time uncertainty (0 when not computed)
  uint16_t mask;    // support of the fitted amplitudes: bit k set when X()[k] > 0
  uint8_t status;
  int outer_iters;
  int fnnls_iters;
  int inner_solves;
  double flops;
};

enum : uint8_t { CH_OK = 0, CH_NNLS_MAXITER = 1, CH_OUTER_MAXITER = 2, CH_NONFINITE = 4, CH_BADINPUT = 8 };

// DoFit, multifit_cpu/src/PulseChiSqSNNLS.cpp:21-147
void dofit(const FitConfig& cfg, const double* samples, double pederr, FitResult& out, bool count) {
  const int N = cfg.N, K = cfg.K;
  FitState S;
  Flops fl;
  Flops* f = count ? &fl : nullptr;
  std::memcpy(S.samp, samples, sizeof(double) * N);
  std::memcpy(S.P, cfg.P, sizeof(double) * N * K);
  for (int k = 0; k < K; ++k) S.amp[k] = 0.;
  S.chisq = 0.;
  S.outer_iters = 0;
  S.nonfinite = 0;
  S.outer_maxed = 0;

  minimize(cfg, pederr, S, f);
  const FnnlsStats main_st = S.st;
  const int main_outer = S.outer_iters;
  const int main_maxed = S.outer_maxed;
  double ampmin[KMAX];
  std::memcpy(ampmin, S.amp, sizeof(double) * K);
  out.err = 0.;

  if (cfg.compute_errors) {
    int kin = -1;
    for (int k = 0; k < K; ++k)
      if (cfg.bxs[k] == 0) { kin = k; break; }
    if (kin >= 0) {
      const double approxerr = approx_uncertainty(cfg, S, kin, f);
      const double chisq0 = S.chisq;
      const double x0 = ampmin[kin];
      double pulse_in[KMAX];
      for (int i = 0; i < N; ++i) { pulse_in[i] = S.P[kin * N + i]; S.P[kin * N + i] = 0.; }
      const double xplus = x0 + approxerr;
      S.amp[kin] = xplus;
      for (int i = 0; i < N; ++i) S.samp[i] = FMA(-xplus, pulse_in[i], samples[i]);
      minimize(cfg, pederr, S, f);
      const double chip = compute_chisq(cfg, S, f);
      const double sigmaplus = std::fabs(xplus - x0) / std::sqrt(chip - chisq0);
      if (x0 / sigmaplus > 0.5) {
        const double xminus = std::max(0., x0 - approxerr);
        S.amp[kin] = xminus;
        for (int i = 0; i < N; ++i) S.samp[i] = FMA(-xminus, pulse_in[i], samples[i]);
        minimize(cfg, pederr, S, f);
        const double chim = compute_chisq(cfg, S, f);
        const double sigmaminus = std::fabs(xminus - x0) / std::sqrt(chim - chisq0);
        out.err = 0.5 * (sigmaplus + sigmaminus);
      } else {
        out.err = sigmaplus;
      }
      S.chisq = chisq0;
    }
  }

  std::memcpy(out.amp, ampmin, sizeof(double) * K);
  for (int k = K; k < KMAX; ++k) out.amp[k] = 0.;
  out.chisq = S.chisq;
  // active set = support of X(): the final FNNLS call of Minimize restarts
  // from an empty passive set and usually stops at once, so its passive set
  // is not the set of fitted pulses.
  uint16_t support = 0;
  for (int k = 0; k < K; ++k)
    if (ampmin[k] > 0.) support |= uint16_t(1u << k);
  out.mask = support;
  uint8_t status = CH_OK;
  if (!main_st.converged) status |= CH_NNLS_MAXITER;
  if (main_maxed) status |= CH_OUTER_MAXITER;
  bool finite = std::isfinite(out.chisq);
  for (int k = 0; k < K; ++k) finite = finite && std::isfinite(out.amp[k]);
  if (!finite) status |= CH_NONFINITE;
  bool bad = !std::isfinite(pederr);
  for (int i = 0; i < N; ++i) bad = bad || !std::isfinite(samples[i]);
  if (bad) status |= CH_BADINPUT;
  out.status = status;
  out.outer_iters = main_outer;
  out.fnnls_iters = main_st.outer_iters;
  out.inner_solves = main_st.inner_solves;
  out.flops = fl.v;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API (ctypes)
// ---------------------------------------------------------------------------
extern "C" {

int oracle_abi_version() { return 1; }

// Linear-algebra primitives on row-major square matrices of leading dim ld.
void oracle_cholesky(const double* M, double* L, int ld, int view) { cholesky_rows(M, L, ld, 0, view, nullptr); }
void oracle_forward(const double* L, int ld, const double* b, double* y, int n) { forward_subst(L, ld, b, y, n, nullptr); }
void oracle_backward(const double* L, int ld, const double* y, double* x, int n) { backward_subst(L, ld, y, x, n, nullptr); }
void oracle_rc_addition(const double* M, double* L, int ld, const double* b, double* y, int view) {
  fused_rc_addition(M, L, ld, b, y, view, nullptr);
}
void oracle_inbetween_removal(const double* M, double* L, int ld, const double* b, double* y, int position, int view) {
  fused_inbetween_removal(M, L, ld, b, y, position, view, nullptr);
}
void oracle_swap_sym(double* M, int ld, int n, int a, int b) { swap_sym(M, ld, n, a, b); }

// FNNLS on a pre-whitened problem. A: N x K column-major. x: warm start in,
// solution out. start: 0 reference, 1 support start. stats: [outer_iters, inner_solves, converged, passive, mask].
void oracle_inplace_fnnls(const double* A, const double* b, double* x, int N, int K, double eps, int max_iter,
                          int variant, int start, int* stats) {
  FnnlsStats st;
  inplace_fnnls(A, b, x, N, K, eps, max_iter, variant, start, &st, nullptr);
  if (stats) {
    stats[0] = st.outer_iters;
    stats[1] = st.inner_solves;
    stats[2] = st.converged;
    stats[3] = st.passive;
    stats[4] = st.mask;
  }
}

// Batch fit with one set of conditions (P, R, fullpulsecov, bxs) shared by all
// channels. samples: [n][sample_stride]; pederr: [n]; outputs: amplitudes
// [n][K], chi2 [n], mask [n], status [n], iters [n][3] (outer, fnnls, inner),
// err [n] (may be null), flops [n] (may be null). nthreads <= 0 uses all cores.
int oracle_fit_batch(int64_t n, int N, int K, const double* samples, int sample_stride, const double* pederr,
                     const double* P, const double* R, const double* fpc, const int8_t* bxs, double eps,
                     int max_iter_nnls, int max_iter_outer, double dchi2_tol, int variant, int start,
                     int compute_errors, int nthreads, double* amplitudes, double* chi2, uint16_t* mask, uint8_t* status,
                     int32_t* iters, double* err, double* flops) {
  if (N < 1 || N > KMAX || K < 1 || K > KMAX || n < 0) return 1;
  int8_t default_bxs[KMAX];
  if (!bxs) {
    for (int k = 0; k < K; ++k) default_bxs[k] = int8_t(k - 5);
    bxs = default_bxs;
  }
  FitConfig cfg{N, K, P, R, fpc, bxs, eps, max_iter_nnls, max_iter_outer, dchi2_tol, variant, start, compute_errors};
  const bool count = flops != nullptr;
  auto work = [&](int64_t lo, int64_t hi) {
    for (int64_t c = lo; c < hi; ++c) {
      FitResult r;
      dofit(cfg, samples + c * sample_stride, pederr[c], r, count);
      for (int k = 0; k < K; ++k) amplitudes[c * K + k] = r.amp[k];
      chi2[c] = r.chisq;
      if (mask) mask[c] = r.mask;
      if (status) status[c] = r.status;
      if (iters) {
        iters[c * 3 + 0] = r.outer_iters;
        iters[c * 3 + 1] = r.fnnls_iters;
        iters[c * 3 + 2] = r.inner_solves;
      }
      if (err) err[c] = r.err;
      if (flops) flops[c] = r.flops;
    }
  };
  int nt = nthreads > 0 ? nthreads : int(std::max(1u, std::thread::hardware_concurrency()));
  if (nt == 1 || n < 2 * nt) {
    work(0, n);
    return 0;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = std::min<int64_t>(n, lo + chunk);
    if (lo < hi) pool.emplace_back(work, lo, hi);
  }
  for (auto& th : pool) th.join();
  return 0;
}

int oracle_hardware_threads() { return int(std::thread::hardware_concurrency()); }

// Independent checks -------------------------------------------------------

// KKT residuals of min ||A x - b||^2, x >= 0, on the unwhitened normal
// equations: g = A^T (A x - b). Returns max over i of
//   |g_i| for x_i > 0 (stationarity), max(0, -g_i) for x_i == 0 (dual feasibility),
//   max(0, -x_i) (primal feasibility), scaled by scale.
double oracle_kkt_violation(const double* A, const double* b, const double* x, int N, int K) {
  double r[KMAX];
  for (int i = 0; i < N; ++i) {
    long double acc = 0;
    for (int k = 0; k < K; ++k) acc += (long double)A[k * N + i] * x[k];
    r[i] = double(acc - b[i]);
  }
  double worst = 0;
  for (int k = 0; k < K; ++k) {
    long double g = 0;
    for (int i = 0; i < N; ++i) g += (long double)A[k * N + i] * r[i];
    double v;
    if (x[k] > 0) v = std::fabs(double(g));
    else v = std::max(0., -double(g));
    v = std::max(v, std::max(0., -x[k]));
    worst = std::max(worst, v);
  }
  return worst;
}

// Exhaustive NNLS: enumerate every passive set, solve the unconstrained
// least squares on it with long-double normal equations, keep feasible
// solutions with the smallest residual. K <= 10 (1024 subsets).
double oracle_nnls_bruteforce(const double* A, const double* b, int N, int K, double* x_out) {
  long double best = std::numeric_limits<long double>::infinity();
  double bestx[KMAX] = {0};
  for (unsigned m = 0; m < (1u << K); ++m) {
    int idx[KMAX], p = 0;
    for (int k = 0; k < K; ++k)
      if (m & (1u << k)) idx[p++] = k;
    long double G[KMAX][KMAX + 1];
    for (int a = 0; a < p; ++a) {
      for (int c = 0; c < p; ++c) {
        long double acc = 0;
        for (int i = 0; i < N; ++i) acc += (long double)A[idx[a] * N + i] * A[idx[c] * N + i];
        G[a][c] = acc;
      }
      long double acc = 0;
      for (int i = 0; i < N; ++i) acc += (long double)A[idx[a] * N + i] * b[i];
      G[a][p] = acc;
    }
    // Gaussian elimination with partial pivoting
    bool ok = true;
    for (int c = 0; c < p && ok; ++c) {
      int piv = c;
      for (int r = c + 1; r < p; ++r)
        if (std::fabs((double)G[r][c]) > std::fabs((double)G[piv][c])) piv = r;
      if (G[piv][c] == 0) { ok = false; break; }
      if (piv != c)
        for (int q = 0; q <= p; ++q) std::swap(G[c][q], G[piv][q]);
      for (int r = c + 1; r < p; ++r) {
        const long double fct = G[r][c] / G[c][c];
        for (int q = c; q <= p; ++q) G[r][q] -= fct * G[c][q];
      }
    }
    if (!ok) continue;
    long double sol[KMAX];
    for (int r = p - 1; r >= 0; --r) {
      long double acc = G[r][p];
      for (int q = r + 1; q < p; ++q) acc -= G[r][q] * sol[q];
      sol[r] = acc / G[r][r];
    }
    bool feas = true;
    for (int a = 0; a < p; ++a) feas = feas && sol[a] > 0;
    if (!feas) continue;
    double xx[KMAX] = {0};
    for (int a = 0; a < p; ++a) xx[idx[a]] = double(sol[a]);
    long double res = 0;
    for (int i = 0; i < N; ++i) {
      long double acc = -b[i];
      for (int k = 0; k < K; ++k) acc += (long double)A[k * N + i] * xx[k];
      res += acc * acc;
    }
    if (res < best) {
      best = res;
      std::memcpy(bestx, xx, sizeof(bestx));
    }
  }
  std::memcpy(x_out, bestx, sizeof(double) * K);
  return double(best);
}

// Lawson-Hanson active-set NNLS (the algorithm of nnls/src/nnls.cpp:15-228,
// restated from its published description; QR replaced by long-double normal
// equations on the passive set). Returns the number of outer iterations.
int oracle_nnls_lawson_hanson(const double* A, const double* b, int N, int K, double* x, int max_iter) {
  bool P[KMAX] = {false};
  for (int k = 0; k < K; ++k) x[k] = 0;
  auto solve_passive = [&](double* z) -> bool {
    int idx[KMAX], p = 0;
    for (int k = 0; k < K; ++k)
      if (P[k]) idx[p++] = k;
    long double G[KMAX][KMAX + 1];
    for (int a = 0; a < p; ++a) {
      for (int c = 0; c < p; ++c) {
        long double acc = 0;
        for (int i = 0; i < N; ++i) acc += (long double)A[idx[a] * N + i] * A[idx[c] * N + i];
        G[a][c] = acc;
      }
      long double acc = 0;
      for (int i = 0; i < N; ++i) acc += (long double)A[idx[a] * N + i] * b[i];
      G[a][p] = acc;
    }
    for (int c = 0; c < p; ++c) {
      int piv = c;
      for (int r = c + 1; r < p; ++r)
        if (std::fabs((double)G[r][c]) > std::fabs((double)G[piv][c])) piv = r;
      if (G[piv][c] == 0) return false;
      if (piv != c)
        for (int q = 0; q <= p; ++q) std::swap(G[c][q], G[piv][q]);
      for (int r = c + 1; r < p; ++r) {
        const long double fct = G[r][c] / G[c][c];
        for (int q = c; q <= p; ++q) G[r][q] -= fct * G[c][q];
      }
    }
    long double sol[KMAX];
    for (int r = p - 1; r >= 0; --r) {
      long double acc = G[r][p];
      for (int q = r + 1; q < p; ++q) acc -= G[r][q] * sol[q];
      sol[r] = acc / G[r][r];
    }
    for (int k = 0; k < K; ++k) z[k] = 0;
    for (int a = 0; a < p; ++a) z[idx[a]] = double(sol[a]);
    return true;
  };
  int it = 0;
  for (; it < max_iter; ++it) {
    // gradient w = A^T (b - A x)
    double r[KMAX], w[KMAX];
    for (int i = 0; i < N; ++i) {
      long double acc = b[i];
      for (int k = 0; k < K; ++k) acc -= (long double)A[k * N + i] * x[k];
      r[i] = double(acc);
    }
    int jmax = -1;
    double wmax = 0;
    double scale = 0;
    for (int k = 0; k < K; ++k) {
      long double acc = 0;
      for (int i = 0; i < N; ++i) acc += (long double)A[k * N + i] * r[i];
      w[k] = double(acc);
      for (int i = 0; i < N; ++i) scale = std::max(scale, std::fabs(A[k * N + i] * b[i]));
    }
    const double tol = 1e-13 * std::max(1.0, scale) * N;
    for (int k = 0; k < K; ++k)
      if (!P[k] && w[k] > tol && (jmax < 0 || w[k] > wmax)) { jmax = k; wmax = w[k]; }
    if (jmax < 0) break;
    P[jmax] = true;
    while (true) {
      double z[KMAX];
      if (!solve_passive(z)) { P[jmax] = false; return it; }
      bool feas = true;
      for (int k = 0; k < K; ++k)
        if (P[k] && z[k] <= 0) feas = false;
      if (feas) {
        for (int k = 0; k < K; ++k) x[k] = z[k];
        break;
      }
      double alpha = 2;
      for (int k = 0; k < K; ++k)
        if (P[k] && z[k] <= 0) alpha = std::min(alpha, x[k] / (x[k] - z[k]));
      for (int k = 0; k < K; ++k) x[k] += alpha * (z[k] - x[k]);
      for (int k = 0; k < K; ++k)
        if (P[k] && x[k] <= 1e-300) { P[k] = false; x[k] = 0; }
    }
  }
  return it;
}

}  // extern "C"
