// Per-channel form of the reduced-precision fit (MF_PREC_MIXED / MF_PREC_FP32)
// for what the passive-set tables cannot serve: a covariance that depends on
// the channel's own amplitudes (a non-zero pulse covariance, updateCov of
// multifit_cpu/src/PulseChiSqSNNLS.cpp:169-194), the MINOS-like in-time
// uncertainty (:75-146, :202-207), and shapes without tables.
//
// One thread per channel runs DoFit (fit_core.cuh). Each Minimize
// (PulseChiSqSNNLS.cpp:149-166) is done in two phases:
//   1. FP32: the outer chi2 loop -- covariance, Cholesky, whitening, the
//      FNNLS with the incremental Cholesky, chi2 -- in float, from the
//      caller's start, to its own convergence (|delta chi2| < tol);
//   2. FP64: the same loop in double, seeded with the FP32 amplitudes and
//      chi2, the FNNLS starting from their support (MF_START_SUPPORT). Its
//      first iteration is the one FP64 covariance factor, refinement solve on
//      the converged passive set and FP64 residual / chi2; when the FP32 phase
//      found the right set and chi2 within tol, the loop stops there.
//      Otherwise it goes on in FP64 -- adding or dropping columns, iterating
//      the covariance -- to the FP64 fixed point, so the result never rests on
//      the FP32 arithmetic: it is the FP64 KKT point of the last covariance,
//      with the reference's stopping rule.
// FP32 is abandoned for a channel whose FP32 phase produced a non-finite
// value (a pivot of the FP32 Cholesky at or below zero): phase 2 then starts
// from the caller's start, as the plain FP64 path does.
//
// Against the FP64 path from a zero start the only difference is where the
// outer loop enters: the fixed point is the same (one more outer iteration
// moves converged amplitudes by < 1e-8 relative on the ECAL fixtures with a
// pulse covariance), so the amplitudes agree to the form's 1e-4 bound.
//
// The lanes of a warp run the FP64 phase together (fit_core.cuh's Minimize
// keeps its outer loop warp-uniform), and the FP32 phase first, so the FP64
// pipe sees convergent warps.
#include "fit_core.cuh"

namespace mfgb {
namespace {

// FNNLS iterations of the FP32 phase (its result only seeds the FP64 phase)
constexpr int kCovIter32 = 3 * KMAX;

template <int NT, int KT, bool C>
__device__ void minimize_cov(const DevConditions& c, const DevOptions& o, int N, int K, double pederr,
                             FitState<double>& S, Counter<C>& f, unsigned lanes) {
  FitState<float> S32;
  bool held[KMAX];  // columns zeroed by the MINOS refits keep their double amplitude
  for (int i = 0; i < N; ++i) S32.samp[i] = float(S.samp[i]);
  for (int k = 0; k < K; ++k) {
    S32.amp[k] = float(S.amp[k]);
    bool zero = true;
    for (int i = 0; i < N; ++i) {
      S32.P[k * N + i] = float(S.P[k * N + i]);
      zero = zero && S.P[k * N + i] == 0.;
    }
    held[k] = zero;
  }
  S32.chisq = float(S.chisq);
  S32.st = FnnlsOut{0, 0, 0, 0};
  S32.outer_iters = 0;
  S32.outer_maxed = 0;
  DevOptions o32 = o;
  o32.max_iter_nnls = kCovIter32;
  o32.nnls_start = MF_START_SUPPORT;
  Counter<false> f32;  // the FP32 phase's flops are not FP64 work
  minimize<NT, KT>(c, o32, N, K, float(pederr), S32, f32, lanes);
  bool good = isfinite(S32.chisq);
  for (int k = 0; k < K; ++k) good = good && isfinite(S32.amp[k]);
  if (good) {
    for (int k = 0; k < K; ++k)
      if (!held[k]) S.amp[k] = double(S32.amp[k]);
    S.chisq = double(S32.chisq);
  }
  DevOptions o64 = o;
  o64.nnls_start = MF_START_SUPPORT;
  minimize<NT, KT>(c, o64, N, K, pederr, S, f, lanes);
}

template <int NT, int KT, bool C>
__global__ void __launch_bounds__(128) fit_cov_kernel(const FitArgs a, int set, int flag_bad) {
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
      mine = t == set;
    }
  }
  const unsigned lanes = __ballot_sync(0xffffffffu, mine);  // taken while the warp is converged
  if (!mine) return;
  const DevConditions& c = a.cond[set];
  const int N = NT > 0 ? NT : c.N;
  const int K = KT > 0 ? KT : c.K;
  Counter<C> f;
  dofit_with<NT, KT, C>(a, c, ch, lanes, f, [&](FitState<double>& S, double pederr, unsigned ln) {
    minimize_cov<NT, KT, C>(c, a.opt, N, K, pederr, S, f, ln);
  });
}

template <bool C>
cudaError_t launch_cov_sets(const FitArgs& a, int block, cudaStream_t s, LaunchTimer* tm) {
  const unsigned grid = unsigned((a.n + block - 1) / block);
  for (int t = 0; t < a.n_ctypes; ++t) {
    const DevConditions& c = a.cond[t];
    const int flag = t == 0;
    if (tm) tm->mark(MF_K_FIT_COV, s);
    if (c.N == 10 && c.K == 10) fit_cov_kernel<10, 10, C><<<grid, block, 0, s>>>(a, t, flag);
    else if (c.N == 8 && c.K == 8) fit_cov_kernel<8, 8, C><<<grid, block, 0, s>>>(a, t, flag);
    else fit_cov_kernel<0, 0, C><<<grid, block, 0, s>>>(a, t, flag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_fit_cov(const FitArgs& a, int block, cudaStream_t s, bool instrumented, LaunchTimer* tm) {
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  return instrumented ? launch_cov_sets<true>(a, block, s, tm) : launch_cov_sets<false>(a, block, s, tm);
}

}  // namespace mfgb
