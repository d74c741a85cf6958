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
__device__ void dofit(const FitArgs& a, const DevConditions& c, int64_t ch, unsigned lanes, double* row) {
  const int N = NT > 0 ? NT : c.N;
  const int K = KT > 0 ? KT : c.K;
  Counter<C> f;
  dofit_with<NT, KT, C, R>(a, c, ch, lanes, f, row, row, KMAX, [&](FitState<double>& S, double pederr, unsigned ln) {
    minimize<NT, KT, C, double, R>(c, a.opt, N, K, pederr, S, f, ln);
  });
}

constexpr int kFitBlock = 128;  // the largest block of the kernel (its launch bound)
// Three blocks of 128 per SM: 168 registers a thread, with which the unrolled
// 10 x 10 fit keeps its working set in registers and its packed arrays in a
// 2.4 KB local frame (left free, the compiler chose 128 registers and spilled
// 2.3 KB); 12 warps per SM keep the FP64 pipe ~90 % busy.
constexpr int kFitBlocksPerSm = 3;

// One launch per condition set (lanes of other sets idle); out-of-range set
// indices are flagged by the first launch. A warp stages its 32 channels'
// samples, and afterwards their amplitudes, through one shared-memory row per
// channel with coalesced loads and stores.
template <int NT, int KT, bool C, bool R = false>
__global__ void __launch_bounds__(kFitBlock, kFitBlocksPerSm) fit_fp64_kernel(const FitArgs a, int set, int flag_bad) {
  __shared__ double stage[kFitBlock * KMAX];
  const int lane = int(threadIdx.x & 31u);
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
  if (lanes == 0u) return;
  const DevConditions& c = a.cond[set];
  const int N = NT > 0 ? NT : c.N;
  const int64_t ch0 = ch - lane;
  const int nw = a.n - ch0 < 32 ? int(a.n - ch0) : 32;  // the warp's channels inside the batch
  double* const rows = stage + (threadIdx.x - lane) * KMAX;
  stage_rows_in(a.samples, a.sample_stride, ch0, nw, N, rows, lane);
  __syncwarp();
  if (mine) dofit<NT, KT, C, R>(a, c, ch, lanes, rows + lane * KMAX);
  __syncwarp();
  // K amplitudes, then zeros up to the row's end or KMAX (amp_stride >= K)
  stage_rows_out(rows, a.amplitudes, a.amp_stride, ch0, nw, a.amp_stride < KMAX ? a.amp_stride : KMAX, lanes, lane);
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
  if (block <= 0) block = kFitBlock;
  if (block > kFitBlock || block % 32) return cudaErrorInvalidConfiguration;
  return instrumented ? launch_sets<true>(a, block, s, tm) : launch_sets<false>(a, block, s, tm);
}

}  // namespace mfgb
