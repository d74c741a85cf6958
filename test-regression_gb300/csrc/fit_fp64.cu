// Plain FP64 multifit: one thread per channel, the whole fit of
// PulseChiSqSNNLS::DoFit (multifit_cpu/src/PulseChiSqSNNLS.cpp:21-147) on the
// device. The FNNLS active-set loop uses the incremental Cholesky of
// inplace_fnnls_test_cholesky (nnls/src/inplace_fnnls_test_cholesky.cu:35-227):
// a row is appended when a column enters the passive set
// (linalgebra/interface/fused_cholesky_substitution.hpp:18-59) and the rows
// from the removal point down are refactored when one leaves (:64-102).
//
// Operation order. Every accumulation is a fused multiply-add with the index
// ascending; triangular solves subtract term by term and divide once by the
// diagonal; division and sqrt are IEEE-754 correctly rounded. This file is
// compiled with --fmad=false so that no other product is fused. The CPU
// oracle computes in the same order, so the two agree bit for bit, and the
// incremental factor equals a fresh factorisation of the passive block
// (which is what the reference's inplace_fnnls refactors on every step).
//
// The FP64 pipe of the GB300 issues about 1/58 of the FP32 rate, so this
// kernel is bound by FP64 instructions; integer, shared-memory and local
// traffic hide under them.
#include "fit_core.cuh"

namespace mfgb {
namespace {

// DoFit with the FP64 Minimize: the plain drop-in (R = false), or the
// per-channel form's FP64 continuation (R = true: the covariance factor's
// diagonal inverted once per row, multiplications for the ~(K + 3) N
// divisions of the factor, whitening and chi2 -- on this GPU an FP64 division
// is a sequence of about ten FP64 instructions).
template <int NT, int KT, bool C, bool R>
__device__ void dofit(const FitArgs& a, const DevConditions& c, int64_t ch, unsigned lanes) {
  const int N = NT > 0 ? NT : c.N;
  const int K = KT > 0 ? KT : c.K;
  Counter<C> f;
  dofit_with<NT, KT, C, R>(a, c, ch, lanes, f, [&](FitState<double>& S, double pederr, unsigned ln) {
    minimize<NT, KT, C, double, R>(c, a.opt, N, K, pederr, S, f, ln);
  });
}

// One launch per condition set (lanes of other sets idle); out-of-range set
// indices are flagged by the first launch.
template <int NT, int KT, bool C, bool R = false>
__global__ void __launch_bounds__(128) fit_fp64_kernel(const FitArgs a, int set, int flag_bad) {
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
  if (mine) dofit<NT, KT, C, R>(a, a.cond[set], ch, lanes);
}

}  // namespace

template <bool C>
cudaError_t launch_sets(const FitArgs& a, int block, cudaStream_t s, LaunchTimer* tm) {
  const unsigned grid = unsigned((a.n + block - 1) / block);
  for (int t = 0; t < a.n_ctypes; ++t) {
    const DevConditions& c = a.cond[t];
    const int flag = t == 0;
    if (tm) tm->mark(MF_K_FIT_FP64, s);
    // the seeded continuation of the per-channel form with reciprocals (its
    // instrumented count runs the division form)
    if (a.seeded && !C && c.N == 10 && c.K == 10) fit_fp64_kernel<10, 10, false, true><<<grid, block, 0, s>>>(a, t, flag);
    else if (a.seeded && !C) fit_fp64_kernel<0, 0, false, true><<<grid, block, 0, s>>>(a, t, flag);
    else if (c.N == 10 && c.K == 10) fit_fp64_kernel<10, 10, C><<<grid, block, 0, s>>>(a, t, flag);
    else if (c.N == 8 && c.K == 8) fit_fp64_kernel<8, 8, C><<<grid, block, 0, s>>>(a, t, flag);
    else fit_fp64_kernel<0, 0, C><<<grid, block, 0, s>>>(a, t, flag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_fit_fp64(const FitArgs& a, int block, cudaStream_t s, bool instrumented, LaunchTimer* tm) {
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  return instrumented ? launch_sets<true>(a, block, s, tm) : launch_sets<false>(a, block, s, tm);
}

}  // namespace mfgb
