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

constexpr int kFitBlock = 128;  // the largest block of the kernel (its launch bound)
// Three blocks of 128 per SM: 168 registers a thread, with which the unrolled
// 10 x 10 fit keeps its working set in registers and its packed arrays in a
// ~2.5 KB local frame (left free, the compiler chose 128 registers and
// spilled 2.3 KB); 12 warps per SM keep the FP64 pipe ~90 % busy.
constexpr int kFitBlocksPerSm = 3;

// DoFit with the FP64 Minimize: the plain drop-in (R = false), or the
// per-channel form's FP64 continuation (R = true: the covariance factor's
// diagonal inverted once per row, multiplications for the ~(K + 3) N
// divisions of the factor, whitening and chi2 -- on this GPU an FP64 division
// is a sequence of about ten FP64 instructions).
//
// One wave of resident warps; warp w fits the channels of condition set `set`
// in [w chunk, (w + 1) chunk), a lane one channel at a time, one outer
// iteration per step (ChannelFit). The warp stages each batch of 32
// channels' samples through one shared-memory row per channel with coalesced
// loads; channels of other sets are skipped (their lanes do not idle through
// another set's fits), those with an out-of-range set index flagged by the
// first launch.
//
// Two ways to hand out channels. A channel's first outer iteration is its
// costliest (its FNNLS starts from x = 0 and adds ~9 columns one by one; the
// later ones, from the previous amplitudes, add ~0.3), so a warp fits the
// first iterations of 32 channels side by side (REFILL = false: new channels
// only once every lane is done). The later iterations (2 or 3 per channel, 3
// in nearly every warp of 32) run with REFILL = true: a lane takes the warp's
// next channel as soon as its own is done, so no lane idles through another
// channel's third iteration. (Refilling the first pass too put a first
// iteration's FNNLS into every step: 27.5 -> 36.5 ms per 1M channels.)
template <int NT, int KT, bool C, bool R, bool REFILL>
__global__ void __launch_bounds__(kFitBlock, kFitBlocksPerSm)
    fit_fp64_kernel(const FitArgs a, int set, int flag_bad, int64_t chunk) {
  __shared__ double stage[kFitBlock * KMAX];
  const int lane = int(threadIdx.x & 31u);
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int64_t next = warp * chunk;  // the warp's next channel to stage
  const int64_t end = next + chunk < a.n ? next + chunk : a.n;
  if (next >= end) return;  // warp-uniform
  const DevConditions& c = a.cond[set];
  const int N = NT > 0 ? NT : c.N;
  double* const rows = stage + (threadIdx.x - lane) * KMAX;
  ChannelFit<NT, KT, C, R> fit;
  bool busy = false;
  unsigned avail = 0u;  // staged channels of this set not taken yet (warp-uniform)
  int64_t sbase = 0;    // first channel of the staged batch
  for (;;) {
    if (busy) busy = fit.prepare(a, c);  // false: the channel is done, its outputs written
    // idle lanes take the staged channels of this set in order, staging the
    // next batch when these run out (without REFILL only once all are idle)
    bool filling = REFILL;
    for (;;) {
      const unsigned idle = __ballot_sync(0xffffffffu, !busy);
      if (idle == 0u) break;
      if (!REFILL && idle == 0xffffffffu) filling = true;
      if (!filling) break;
      if (avail == 0u) {
        if (next >= end) break;
        const int nw = end - next < 32 ? int(end - next) : 32;
        __syncwarp();  // every lane has copied its row of the previous batch
        stage_rows_in(a.samples, a.sample_stride, next, nw, N, rows, lane);
        bool mine = false;
        if (lane < nw) {
          const int64_t ch = next + lane;
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
        avail = __ballot_sync(0xffffffffu, mine);
        sbase = next;
        next += nw;
        __syncwarp();  // the staged rows are visible to every lane
        continue;
      }
      const int navail = __popc(avail);
      const int rank = __popc(idle & ((1u << lane) - 1u));  // among the idle lanes
      if (!busy && rank < navail) {
        unsigned m = avail;
        for (int r = 0; r < rank; ++r) m &= m - 1u;  // drop the lower `rank` channels
        const int row = __ffs(int(m)) - 1;
        fit.start(a, c, sbase + row, rows + row * KMAX);
        busy = fit.prepare(a, c);
      }
      const int taken = __popc(idle) < navail ? __popc(idle) : navail;
      for (int r = 0; r < taken; ++r) avail &= avail - 1u;
    }
    const unsigned act = __ballot_sync(0xffffffffu, busy);
    if (act == 0u) break;
    if (busy) fit.iterate(a, c, act);
  }
}

}  // namespace

template <bool C, bool REFILL>
cudaError_t launch_pass(const FitArgs& a, int t, unsigned grid, int block, int64_t chunk, cudaStream_t s) {
  const DevConditions& c = a.cond[t];
  const int flag = t == 0;
  // the per-channel form's continuation with reciprocals (its instrumented
  // count runs the division form); it always refills
  if constexpr (REFILL && !C) {
    if (a.seeded == 1) {
      if (c.N == 10 && c.K == 10) fit_fp64_kernel<10, 10, false, true, true><<<grid, block, 0, s>>>(a, t, flag, chunk);
      else fit_fp64_kernel<0, 0, false, true, true><<<grid, block, 0, s>>>(a, t, flag, chunk);
      return cudaGetLastError();
    }
  }
  if (c.N == 10 && c.K == 10) fit_fp64_kernel<10, 10, C, false, REFILL><<<grid, block, 0, s>>>(a, t, flag, chunk);
  else if (c.N == 8 && c.K == 8) fit_fp64_kernel<8, 8, C, false, REFILL><<<grid, block, 0, s>>>(a, t, flag, chunk);
  else fit_fp64_kernel<0, 0, C, false, REFILL><<<grid, block, 0, s>>>(a, t, flag, chunk);
  return cudaGetLastError();
}

// Per condition set: the first outer iteration of every channel in lockstep,
// then the rest of the fit (later iterations, error refits) with refill,
// seeded from the first pass's outputs. A fit of one outer iteration at most,
// and the per-channel form's continuation (seeded already), run in one pass.
template <bool C>
cudaError_t launch_sets(const FitArgs& a, int block, cudaStream_t s, LaunchTimer* tm) {
  // one wave of resident blocks, the channels split evenly over its warps
  const int64_t resident = int64_t(a.sms > 0 ? a.sms : 1) * kFitBlocksPerSm * (kFitBlock / block);
  const int64_t needed = (a.n + block - 1) / block;
  const unsigned grid = unsigned(needed < resident ? needed : resident);
  const int64_t warps = int64_t(grid) * (block / 32);
  const int64_t chunk = (a.n + warps - 1) / warps;
  const bool two_pass = !a.seeded && a.opt.max_iter_outer > 1;
  FitArgs first = a;
  first.opt.max_iter_outer = 1;
  first.opt.compute_errors = 0;
  FitArgs rest = a;
  rest.seeded = 2;
  for (int t = 0; t < a.n_ctypes; ++t) {
    cudaError_t e;
    if (two_pass) {
      if (tm) tm->mark(MF_K_FIT_FP64, s);
      e = launch_pass<C, false>(first, t, grid, block, chunk, s);
      if (e != cudaSuccess) return e;
      if (tm) tm->mark(MF_K_FIT_FP64, s);
      e = launch_pass<C, true>(rest, t, grid, block, chunk, s);
    } else {
      if (tm) tm->mark(MF_K_FIT_FP64, s);
      e = a.seeded ? launch_pass<C, true>(a, t, grid, block, chunk, s) : launch_pass<C, false>(a, t, grid, block, chunk, s);
    }
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
