// The FP64 drop-in's per-channel routines (test-regression_gb300/csrc/
// fit_core.cuh) compiled for the host, so that the CPU suite checks the
// kernel's own arithmetic, storage and schedule against the oracle and the
// golden fixtures without a GPU. run_warp() is fit_fp64_kernel's warp loop
// with its 32 lanes in lockstep: the code between two ballots of the kernel
// is independent across lanes, so running it for lane 0, 1, ..., 31 in turn
// and forming each ballot from all lanes' values gives the warp's result
// (which lane takes which channel, when the next batch is staged).
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

int popc(unsigned m) { return __builtin_popcount(m); }

// fit_fp64_kernel's loop for the warp fitting set `set` in [next, end)
template <int NT, int KT, bool C, bool R, bool REFILL>
void run_warp(const FitArgs& a, int set, int flag_bad, int64_t next, int64_t end) {
  const DevConditions& c = a.cond[set];
  const int N = NT > 0 ? NT : c.N;
  std::vector<double> rows(32 * KMAX, NAN);
  std::vector<ChannelFit<NT, KT, C, R>> fit(32);
  bool busy[32] = {};
  unsigned avail = 0u;
  int64_t sbase = 0;
  for (;;) {
    for (int l = 0; l < 32; ++l)
      if (busy[l]) busy[l] = fit[l].prepare(a, c);
    bool filling = REFILL;
    for (;;) {
      unsigned idle = 0u;
      for (int l = 0; l < 32; ++l)
        if (!busy[l]) idle |= 1u << l;
      if (idle == 0u) break;
      if (!REFILL && idle == 0xffffffffu) filling = true;
      if (!filling) break;
      if (avail == 0u) {
        if (next >= end) break;
        const int nw = end - next < 32 ? int(end - next) : 32;
        for (int l = 0; l < 32; ++l) stage_rows_in(a.samples, a.sample_stride, next, nw, N, rows.data(), l);
        unsigned mine = 0u;
        for (int l = 0; l < nw; ++l) {
          const int64_t ch = next + l;
          const int t = a.ctype ? int(a.ctype[ch]) : 0;
          if (t >= a.n_ctypes) {
            if (flag_bad) {
              if (a.status) a.status[ch] = CH_BADINPUT;
              a.chi2[ch] = 0.;
            }
          } else if (t == set) {
            mine |= 1u << l;
          }
        }
        avail = mine;
        sbase = next;
        next += nw;
        continue;
      }
      const int navail = popc(avail);
      for (int l = 0; l < 32; ++l) {
        const int rank = popc(idle & ((1u << l) - 1u));
        if (!busy[l] && rank < navail) {
          unsigned m = avail;
          for (int r = 0; r < rank; ++r) m &= m - 1u;
          const int row = __builtin_ctz(m);
          fit[l].start(a, c, sbase + row, rows.data() + row * KMAX);
          busy[l] = fit[l].prepare(a, c);
        }
      }
      const int taken = popc(idle) < navail ? popc(idle) : navail;
      for (int r = 0; r < taken; ++r) avail &= avail - 1u;
    }
    unsigned act = 0u;
    for (int l = 0; l < 32; ++l)
      if (busy[l]) act |= 1u << l;
    if (act == 0u) break;
    for (int l = 0; l < 32; ++l)
      if (busy[l]) fit[l].iterate(a, c, act);
  }
}

template <bool C, bool R, bool REFILL>
void pass(const FitArgs& a, bool generic, int64_t chunk) {
  const int N = a.cond[0].N, K = a.cond[0].K;
  for (int64_t w0 = 0; w0 < a.n; w0 += chunk) {
    const int64_t w1 = w0 + chunk < a.n ? w0 + chunk : a.n;
    if (!generic && N == 10 && K == 10) run_warp<10, 10, C, R, REFILL>(a, 0, 1, w0, w1);
    else if (!generic && N == 8 && K == 8) run_warp<8, 8, C, R, REFILL>(a, 0, 1, w0, w1);
    else run_warp<0, 0, C, R, REFILL>(a, 0, 1, w0, w1);
  }
}

// launch_sets' passes: the first outer iteration of every channel in
// lockstep, then the rest with refill, seeded from the first pass's outputs
template <bool C, bool R>
void dispatch(const FitArgs& a, bool generic, int64_t chunk) {
  if (!a.seeded && a.opt.max_iter_outer > 1) {
    FitArgs* first = new FitArgs(a);
    first->opt.max_iter_outer = 1;
    first->opt.compute_errors = 0;
    pass<C, R, false>(*first, generic, chunk);
    FitArgs* rest = new FitArgs(a);
    rest->seeded = 2;
    pass<C, R, true>(*rest, generic, chunk);
    delete first;
    delete rest;
  } else if (a.seeded) {
    pass<C, R, true>(a, generic, chunk);
  } else {
    pass<C, R, false>(a, generic, chunk);
  }
}

}  // namespace

// Fits n channels of one condition set (mf_conditions layout) with the
// kernel's routines, `chunk` channels per warp. flags: 1 count flops, 2
// reciprocal variant (the per-channel form's continuation), 4 generic-shape
// instantiation, 8 seeded (amplitudes, chi2 and status hold the first outer
// iteration on entry). ctype (or null): each channel's condition set; those
// of set 1 belong to another launch, those of set 2 or above are flagged.
// max_iter_outer: Minimize's iteration cap (50 in the reference).
extern "C" int fit_core_host(const mf_conditions* cond, const double* samples, int sample_stride,
                             const double* pederr, const uint8_t* ctype, int64_t n, int nnls_start, int max_iter_nnls,
                             int compute_errors, int flags, int64_t chunk, int max_iter_outer, double* amplitudes,
                             int amp_stride, double* chi2,
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
  a->cond[1] = a->cond[0];
  a->n_ctypes = ctype ? 2 : 1;
  a->ctype = ctype;
  a->opt.max_iter_nnls = max_iter_nnls;
  a->opt.max_iter_outer = max_iter_outer;
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
  if (chunk < 1) chunk = 1;
  if (flags & 1) dispatch<true, false>(*a, generic, chunk);
  else if (flags & 2) dispatch<false, true>(*a, generic, chunk);
  else dispatch<false, false>(*a, generic, chunk);
  std::free(a);
  return 0;
}
