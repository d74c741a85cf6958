// The FP64 drop-in's per-channel routines (test-regression_gb300/csrc/
// fit_core.cuh) compiled for the host, so that the CPU suite checks the
// kernel's own arithmetic and storage against the oracle and the golden
// fixtures without a GPU. The warp-level pieces run one lane at a time: the
// ballots of a single lane, and the kernel's coalesced staging of samples and
// amplitudes through a warp's shared-memory rows, lane by lane over a
// 32-channel block (each lane's part of a staging loop is independent of the
// others, so running the lanes in turn gives the warp's result).
//
// Built by tests/test_fit_core_host.py with g++ -ffp-contract=off: fma(),
// division and sqrt are IEEE-754 on the host as on the GPU, and nothing else
// fuses, as the kernel's --fmad=false build.
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

using std::isfinite;
static inline unsigned __ballot_sync(unsigned, bool p) { return p ? 1u : 0u; }
static inline void __syncwarp(unsigned = 0xffffffffu) {}

#include "fit_core.cuh"

using namespace mfgb;

namespace {

// The kernel's body for one condition set, a warp (32 channels) at a time;
// `skip_every` > 0 leaves every skip_every-th channel to "another set": it is
// neither fitted nor written.
template <int NT, int KT, bool C, bool R>
void run(const FitArgs& a, int skip_every) {
  const DevConditions& c = a.cond[0];
  const int N = NT > 0 ? NT : c.N;
  const int K = KT > 0 ? KT : c.K;
  std::vector<double> rows(32 * KMAX);
  for (int64_t ch0 = 0; ch0 < a.n; ch0 += 32) {
    const int nw = a.n - ch0 < 32 ? int(a.n - ch0) : 32;
    std::fill(rows.begin(), rows.end(), NAN);
    for (int lane = 0; lane < 32; ++lane) stage_rows_in(a.samples, a.sample_stride, ch0, nw, N, rows.data(), lane);
    unsigned sel = 0;
    for (int lane = 0; lane < nw; ++lane) {
      if (skip_every > 0 && (ch0 + lane) % skip_every == skip_every - 1) continue;
      sel |= 1u << lane;
      double* row = rows.data() + lane * KMAX;
      Counter<C> f;
      dofit_with<NT, KT, C, R>(a, c, ch0 + lane, 1u, f, row, row, KMAX,
                               [&](FitState<double>& S, double pederr, unsigned ln) {
                                 minimize<NT, KT, C, double, R>(c, a.opt, N, K, pederr, S, f, ln);
                               });
    }
    const int width = a.amp_stride < KMAX ? a.amp_stride : KMAX;
    for (int lane = 0; lane < 32; ++lane)
      stage_rows_out(rows.data(), a.amplitudes, a.amp_stride, ch0, nw, width, sel, lane);
  }
}

template <bool C, bool R>
void dispatch(const FitArgs& a, bool generic, int skip_every) {
  const int N = a.cond[0].N, K = a.cond[0].K;
  if (!generic && N == 10 && K == 10) run<10, 10, C, R>(a, skip_every);
  else if (!generic && N == 8 && K == 8) run<8, 8, C, R>(a, skip_every);
  else run<0, 0, C, R>(a, skip_every);
}

}  // namespace

// Fits n channels of one condition set (mf_conditions layout) with the
// kernel's routines. flags: 1 count flops, 2 reciprocal variant (the
// per-channel form's continuation), 4 generic-shape instantiation, 8 seeded
// (amplitudes, chi2 and status hold the first outer iteration on entry).
extern "C" int fit_core_host(const mf_conditions* cond, const double* samples, int sample_stride,
                             const double* pederr, int64_t n, int nnls_start, int max_iter_nnls, int compute_errors,
                             int flags, int skip_every, double* amplitudes, int amp_stride, double* chi2,
                             double* intime, double* errors, uint16_t* active_mask, uint8_t* status, int32_t* iters,
                             double* flops) {
  const int N = cond->nsamples, K = cond->npulses;
  if (N < 1 || N > KMAX || K < 1 || K > KMAX || sample_stride < N || amp_stride < K) return 1;
  FitArgs* a = static_cast<FitArgs*>(std::calloc(1, sizeof(FitArgs)));
  if (!a) return 2;
  DevConditions* d = &a->cond[0];
  d->N = N;
  d->K = K;
  d->intime_col = -1;
  for (int k = 0; k < K; ++k) {
    d->bxs[k] = cond->bxs[k];
    if (d->intime_col < 0 && cond->bxs[k] == 0) d->intime_col = k;
  }
  for (int i = 0; i < N * K; ++i) d->P[i] = cond->pulse_matrix[i];
  for (int i = 0; i < N * N; ++i) d->R[i] = cond->noise_cor[i];
  d->has_fpc = cond->has_fullpulsecov ? 1 : 0;
  if (d->has_fpc) std::memcpy(d->fpc, cond->fullpulsecov, sizeof(double) * (N + 9) * (N + 9));
  a->n_ctypes = 1;
  a->opt.max_iter_nnls = max_iter_nnls;
  a->opt.max_iter_outer = 50;
  a->opt.dchi2_tol = 1e-3;
  a->opt.nnls_eps = 1e-11;
  a->opt.nnls_start = nnls_start;
  a->opt.compute_errors = compute_errors;
  a->n = n;
  a->sample_stride = sample_stride;
  a->amp_stride = amp_stride;
  a->samples = samples;
  a->pederr = pederr;
  a->amplitudes = amplitudes;
  a->chi2 = chi2;
  a->intime = intime;
  a->errors = errors;
  a->active_mask = active_mask;
  a->status = status;
  a->iters = iters;
  a->flops = flops;
  a->seeded = (flags & 8) ? 1 : 0;
  const bool generic = (flags & 4) != 0;
  if (flags & 1) dispatch<true, false>(*a, generic, skip_every);
  else if (flags & 2) dispatch<false, true>(*a, generic, skip_every);
  else dispatch<false, false>(*a, generic, skip_every);
  std::free(a);
  return 0;
}
