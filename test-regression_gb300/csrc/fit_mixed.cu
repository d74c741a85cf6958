// Mixed-precision multifit: an FP32 active-set search and an FP64 (or
// double-float) judge in separate kernels, started cold or from the passive
// sets and amplitudes the warm-start MLP predicted.
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
//   screen_kernel  (cold starts; FP32, branch-free): the residual of the FP32
//     solution in double-float and the KKT test of every inactive column; a
//     channel with provably violating columns is queued for the fix.
//   judge_kernel   (FP64 -- or, for MF_PREC_FP32, the same steps in double-float
//     FP32 arithmetic; lean, branch-free: every lane the same instructions):
//     y, the solve on the passive set through the operator table, the
//     residual, chi2 = ||y - G x||^2 / pederr^2, and the KKT test
//     max w < eps * pederr^2 (the reference's absolute eps on the
//     pederr-scaled gradient, PulseChiSqSNNLS.cpp:242) screened in FP32 with
//     a rounding bound. On warm starts a channel whose amplitudes are positive
//     but whose columns provably violate the test is queued for the fix;
//   fix_kernel     (FP32, compacted): the FNNLS step with those columns and a
//     double-float screen of the new set, then (warm starts)
//   judge_fixed_kernel: the judge again, on the fixed channels only. Every
//     other rejected channel is queued for
//   repair_kernel  (FP64): the FNNLS loop in FP64 to the FP64 KKT point, so
//     the result is the FP64 KKT point whatever the FP32 search found.
// Order per set: cold search, screen, fix, judge, repair; warm search, judge,
// fix, judge_fixed, repair (launch_set).
//
// Why separate kernels: on this GPU an FP64 warp instruction costs the full
// pipe time whatever the number of active lanes, and FP64 results have long
// latency. With the search in the same kernel its register budget (168) left
// three warps per scheduler and the judge's dependent FP64 chains were
// latency-bound (~6x its pipe time). Apart, the judge runs convergent at high
// occupancy, and the queue kernels run their rare channels in full warps; the
// hand-off costs ~124 bytes per channel of HBM traffic.
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
// The search, the screen and the double-float judge take their condition set
// as a kernel parameter of its own (T): its whitening and G entries then sit
// at fixed offsets of the parameter bank and enter the FMAs as immediate
// operands, where a.tab[set] with a run-time set costs an indexed constant
// load per entry (ADU pipe 29 % busy in the judge). Measured per 10M ECAL
// channels: judge 3.02 -> 2.77 ms, screen 1.60 -> 1.50 ms. The fix, the FP64
// judge and the repair read a.tab[set]: with immediate operands the compiler's
// schedule spilled (FP64 judge) or doubled the fix's registers (116 -> 232),
// both slower.
// The search (72 registers unbounded) and the fix (116) are latency-bound on
// their table rows and gathered channels: capped at 64 and 85 registers they
// keep 8 and 6 blocks per SM resident (a few bytes spilled), which cut the
// cold FP32 fit of 10M ECAL channels from 9.53 to 8.97 ms (search 2.83 ->
// 2.69, fix 2.65 -> 2.23 ms).
template <int N, int K, bool WARM>
__global__ void __launch_bounds__(128, 8) search_kernel(const __grid_constant__ MixedArgs a,
                                                          const __grid_constant__ DevMixed T, int set) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (ch == 0) {  // the screen and judge launches that follow fill the fix and repair queues
    a.ws_qcount[0] = 0u;
    a.ws_qcount[1] = 0u;
  }
  if (ch >= a.n) return;
  const int t = a.ctype ? int(a.ctype[ch]) : 0;
  if (t != set) return;
  search_body<N, K, WARM>(a, T, ch);
}

template <int N, int K>
__global__ void __launch_bounds__(128, 6) fix_kernel(const MixedArgs a, int set, int rounds) {
  const DevMixed& T = a.tab[set];
  const unsigned cnt = a.ws_qcount[1];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    fix_body<N, K>(a, T, unsigned(a.ws_fixq[i]), rounds);
}

// The second judge pass: the channels the fix changed (failures go to repair).
template <int N, int K, bool DF>
__global__ void __launch_bounds__(128, DF ? 4 : 6) judge_fixed_kernel(const __grid_constant__ MixedArgs a,
                                                                          const __grid_constant__ DevMixed T, int set) {
  const unsigned cnt = a.ws_qcount[1];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const int64_t ch = int64_t(unsigned(a.ws_fixq[i]));
    if constexpr (DF) judge_df_body<N, K>(a, T, ch, a.ws_qcount, nullptr);
    else judge_body<N, K>(a, a.tab[set], ch, a.ws_qcount, nullptr);
  }
}

template <int N, int K>
__global__ void __launch_bounds__(128) screen_kernel(const __grid_constant__ MixedArgs a,
                                                          const __grid_constant__ DevMixed T, int set) {
  const int64_t ch = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (ch >= a.n) return;
  const int t = a.ctype ? int(a.ctype[ch]) : 0;
  if (t != set) return;
  screen_body<N, K>(a, T, ch, a.ws_qcount + 1);
}

template <int N, int K, bool DF>
__global__ void __launch_bounds__(128, DF ? 4 : 6) judge_kernel(const __grid_constant__ MixedArgs a,
                                                                    const __grid_constant__ DevMixed T, int set,
                                                                    int flag_bad, int fixq) {
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
  unsigned* fix_count = fixq ? a.ws_qcount + 1 : nullptr;
  if constexpr (DF) judge_df_body<N, K>(a, T, ch, a.ws_qcount, fix_count);
  else judge_body<N, K>(a, a.tab[set], ch, a.ws_qcount, fix_count);
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

// The kernels of one condition set. Cold starts: search, screen (queues the
// channels with provably missing columns), fix, judge, repair. Warm starts
// (few channels need a column): search, judge (queues them itself), fix,
// second judge on the fixed channels, repair.
template <int N, int K>
void launch_set(const MixedArgs& a, int t, bool warm, int flag_bad, unsigned grid, unsigned jgrid, unsigned rgrid,
                int block, cudaStream_t s, LaunchTimer* tm) {
  auto mark = [&](int k) {
    if (tm) tm->mark(k, s);
  };
  mark(MF_K_SEARCH);
  if constexpr (N == 10 && K == 10) {
    if (warm) search_kernel<N, K, true><<<grid, block, 0, s>>>(a, a.tab[t], t);
    else search_kernel<N, K, false><<<grid, block, 0, s>>>(a, a.tab[t], t);
  } else {
    search_kernel<N, K, false><<<grid, block, 0, s>>>(a, a.tab[t], t);
  }
  if (!warm) {
    mark(MF_K_SCREEN);
    screen_kernel<N, K><<<jgrid, 128, 0, s>>>(a, a.tab[t], t);
    mark(MF_K_FIX);
    fix_kernel<N, K><<<jgrid, 128, 0, s>>>(a, t, 2);
  }
  mark(MF_K_JUDGE);
  if (a.judge_df) judge_kernel<N, K, true><<<jgrid, 128, 0, s>>>(a, a.tab[t], t, flag_bad, warm ? 1 : 0);
  else judge_kernel<N, K, false><<<jgrid, 128, 0, s>>>(a, a.tab[t], t, flag_bad, warm ? 1 : 0);
  if (warm) {
    // the warm queues hold a few per cent of the channels: one resident wave
    // of blocks strides over them (fix 0.41 -> 0.37 ms, second judge 0.48 ->
    // 0.47 ms per 10M), where a grid over every channel spent its time on
    // blocks that exit at once. The cold fix queue (a quarter of the
    // channels) keeps the full grid: one wave striding was 0.19 ms slower.
    const unsigned sms = unsigned(a.sms > 0 ? a.sms : 1);
    const unsigned fgrid = jgrid < 6 * sms ? jgrid : 6 * sms;
    const unsigned rjgrid = jgrid < (a.judge_df ? 4 : 6) * sms ? jgrid : (a.judge_df ? 4 : 6) * sms;
    mark(MF_K_FIX);
    fix_kernel<N, K><<<fgrid, 128, 0, s>>>(a, t, 1);
    mark(MF_K_REJUDGE);
    if (a.judge_df) judge_fixed_kernel<N, K, true><<<rjgrid, 128, 0, s>>>(a, a.tab[t], t);
    else judge_fixed_kernel<N, K, false><<<rjgrid, 128, 0, s>>>(a, a.tab[t], t);
  }
  mark(MF_K_REPAIR);
  repair_kernel<N, K><<<rgrid, 128, 0, s>>>(a, t);
}

}  // namespace

// The kernels of every condition set in turn (launch_set) (lanes of other sets return at
// once); out-of-range set indices are flagged by the first judge launch.
cudaError_t launch_fit_mixed(const MixedArgs& a, int block, cudaStream_t s, LaunchTimer* tm) {
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  const unsigned grid = unsigned((a.n + block - 1) / block);
  const unsigned jgrid = unsigned((a.n + 127) / 128);
  // the fix and second judge take one thread per queue slot (the queue's
  // worst case is every channel; threads past its length exit at once): their
  // work is gathered and latency-bound, so it wants every thread resident at
  // once. The repair grid is at most eight 128-thread blocks per SM, striding.
  const int64_t rmax = int64_t(a.sms > 0 ? a.sms : 1) * 8;
  const unsigned rgrid = unsigned(jgrid < rmax ? jgrid : rmax);
  int flag_bad = 1;
  for (int t = 0; t < a.n_ctypes; ++t) {
    const DevMixed& T = a.tab[t];
    const bool warm = a.warm_mask && t == a.warm_set;
    if (T.N == 10 && T.K == 10) {
      launch_set<10, 10>(a, t, warm, flag_bad, grid, jgrid, rgrid, block, s, tm);
    } else if (T.N == 8 && T.K == 8 && !warm) {
      launch_set<8, 8>(a, t, false, flag_bad, grid, jgrid, rgrid, block, s, tm);
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
