// Mixed-precision multifit: an FP32 active-set search and an FP64 judge, as
// two kernels, started cold or from the passive sets and amplitudes the
// warm-start MLP predicted.
//
// With an amplitude-independent covariance the whitened problem of a channel
// is min ||G x - y||^2 with the condition set's shared G = L_R^-1 P and
// y = L_R^-1 s (tables.cu); every passive-set solve is x_S = G_S^+ y from the
// set's operator table.
//
//   search_kernel  (FP32, register-heavy, divergent): the FNNLS active-set
//     loop of nnls/src/inplace_fnnls.cu:127-231 -- add the column of largest
//     gradient w = G^T y - H x, solve the passive set, step back and drop
//     columns that go non-positive -- from an empty set or the predicted one;
//     writes the passive mask and the FP32 amplitudes of each channel.
//   screen_kernel  (FP32, branch-free): the accurate KKT screen of the
//     search's set in double-float arithmetic; queues the channels with
//     columns the FP32 search missed for
//   fix_kernel     (FP32, compacted): their FNNLS step and one more screen,
//     so that few channels need the FP64 repair.
//   judge_kernel   (FP64 -- or, for MF_PREC_FP32, the same steps in double-float
//     FP32 arithmetic; lean, branch-free: every lane the same FP64
//     instructions): y in FP64, the FP64 solve on the FP32 passive set, the
//     FP64 residual, chi2 = ||y - G x||^2 / pederr^2, and the KKT test
//     max w < eps * pederr^2 (the reference's absolute eps on the
//     pederr-scaled gradient, PulseChiSqSNNLS.cpp:242) screened in FP32 with
//     a rounding bound. A channel the screen cannot pass (or whose FP64
//     amplitudes are not positive) is queued for
//   repair_kernel  (FP64): the FNNLS loop in FP64 to the FP64 KKT point, so
//     the result is the FP64 KKT point whatever the FP32 search found.
//
// Why two kernels: on this GPU an FP64 warp instruction costs the full pipe
// time whatever the number of active lanes, and FP64 results have long
// latency. In one kernel the FP32 search set the register budget (168), so
// only three warps per scheduler were resident and the dependent FP64 chains
// of the judge were latency-bound (the judge took ~6x its pipe time). Apart,
// the judge runs convergent at high occupancy; the hand-off costs ~124 bytes
// per channel of HBM traffic.
//
// The covariance does not depend on the amplitudes (no fullpulsecov), so the
// outer chi2 loop of Minimize (multifit_cpu/src/PulseChiSqSNNLS.cpp:149-166)
// would only repeat a KKT-converged fit and confirm delta chi2 = 0: this form
// runs it once.
#include "mixed_device.cuh"

namespace mfgb {
namespace {

// ---------------------------------------------------------------------------
// Grid schedule: one thread per channel of the chunk, one launch per kernel
// and condition set (lanes of other sets return at once)
// ---------------------------------------------------------------------------
template <int N, int K, bool WARM>
__global__ void __launch_bounds__(128) search_kernel(const MixedArgs a, int set) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (ch == 0) {  // the screen and judge launches that follow fill the fix and repair queues
    a.ws_qcount[0] = 0u;
    a.ws_qcount[1] = 0u;
  }
  if (ch >= a.n) return;
  const int t = a.ctype ? int(a.ctype[ch]) : 0;
  if (t != set) return;
  search_body<N, K, WARM>(a, a.tab[set], ch);
}

template <int N, int K>
__global__ void __launch_bounds__(128) screen_kernel(const MixedArgs a, int set) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (ch >= a.n) return;
  const int t = a.ctype ? int(a.ctype[ch]) : 0;
  if (t != set) return;
  screen_body<N, K>(a, a.tab[set], ch, a.ws_qcount + 1);
}

template <int N, int K>
__global__ void __launch_bounds__(128) fix_kernel(const MixedArgs a, int set) {
  const DevMixed& T = a.tab[set];
  const unsigned cnt = a.ws_qcount[1];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    fix_body<N, K>(a, T, unsigned(a.ws_queue[i]));
}

template <int N, int K, bool DF>
__global__ void __launch_bounds__(128, DF ? 4 : 6) judge_kernel(const MixedArgs a, int set, int flag_bad) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (ch >= a.n) return;
  const int t = a.ctype ? int(a.ctype[ch]) : 0;
  if (t >= a.n_ctypes) {
    if (flag_bad) {
      if (a.status) a.status[ch] = CH_BADINPUT;
      a.chi2[ch] = 0.;
    }
    return;
  }
  if (t != set) return;
  if constexpr (DF) judge_df_body<N, K>(a, a.tab[set], ch, a.ws_qcount);
  else judge_body<N, K>(a, a.tab[set], ch, a.ws_qcount);
}

// Channels the judge queued, in full warps: an FP64 warp instruction costs the
// same with one active lane as with 32, so a repair left inside the judge
// would cost its whole warp the repair's FP64 time.
template <int N, int K>
__global__ void __launch_bounds__(128) repair_kernel(const MixedArgs a, int set) {
  const DevMixed& T = a.tab[set];
  const unsigned cnt = a.ws_qcount[0];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    judge_repair<N, K>(a, T, int64_t(a.ws_queue[i]));
}

}  // namespace

// One search, screen, fix, judge and repair launch per condition set (lanes of other sets return at
// once); out-of-range set indices are flagged by the first judge launch.
cudaError_t launch_fit_mixed(const MixedArgs& a, int block, cudaStream_t s, LaunchTimer* tm) {
  auto mark = [&](int k) {
    if (tm) tm->mark(k, s);
  };
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  const unsigned grid = unsigned((a.n + block - 1) / block);
  const unsigned jgrid = unsigned((a.n + 127) / 128);
  // the repair grid covers the queue's worst case (every channel) with at most
  // eight 128-thread blocks per SM, striding when the queue is longer
  const int64_t rmax = int64_t(a.sms > 0 ? a.sms : 1) * 8;
  const unsigned rgrid = unsigned(jgrid < rmax ? jgrid : rmax);
  int flag_bad = 1;
  for (int t = 0; t < a.n_ctypes; ++t) {
    const DevMixed& T = a.tab[t];
    const bool warm = a.warm_mask && t == a.warm_set;
    if (T.N == 10 && T.K == 10) {
      mark(MF_K_SEARCH);
      if (warm) search_kernel<10, 10, true><<<grid, block, 0, s>>>(a, t);
      else search_kernel<10, 10, false><<<grid, block, 0, s>>>(a, t);
      mark(MF_K_SCREEN);
      screen_kernel<10, 10><<<jgrid, 128, 0, s>>>(a, t);
      mark(MF_K_FIX);
      fix_kernel<10, 10><<<rgrid, 128, 0, s>>>(a, t);
      mark(MF_K_JUDGE);
      if (a.judge_df) judge_kernel<10, 10, true><<<jgrid, 128, 0, s>>>(a, t, flag_bad);
      else judge_kernel<10, 10, false><<<jgrid, 128, 0, s>>>(a, t, flag_bad);
      mark(MF_K_REPAIR);
      repair_kernel<10, 10><<<rgrid, 128, 0, s>>>(a, t);
    } else if (T.N == 8 && T.K == 8) {
      mark(MF_K_SEARCH);
      search_kernel<8, 8, false><<<grid, block, 0, s>>>(a, t);
      mark(MF_K_SCREEN);
      screen_kernel<8, 8><<<jgrid, 128, 0, s>>>(a, t);
      mark(MF_K_FIX);
      fix_kernel<8, 8><<<rgrid, 128, 0, s>>>(a, t);
      mark(MF_K_JUDGE);
      if (a.judge_df) judge_kernel<8, 8, true><<<jgrid, 128, 0, s>>>(a, t, flag_bad);
      else judge_kernel<8, 8, false><<<jgrid, 128, 0, s>>>(a, t, flag_bad);
      mark(MF_K_REPAIR);
      repair_kernel<8, 8><<<rgrid, 128, 0, s>>>(a, t);
    } else {
      return cudaErrorInvalidValue;
    }
    flag_bad = 0;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace mfgb
