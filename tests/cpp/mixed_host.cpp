// The mixed and FP32 precisions' device routines (test-regression_gb300/csrc/
// mixed_device.cuh) and their passive-set tables (csrc/tables.cu) compiled
// for the host, so that the CPU suite runs the cold-start pipeline of the
// grid schedule -- FP32 search, double-float KKT screen, FP32 fix, the FP64
// or double-float judge, FP64 repair -- channel by channel, queues included,
// without a GPU. Driven by tests/test_mixed_host.py.
//
// The CUDA intrinsics the routines use get host stand-ins below: the
// round-to-nearest single operations are the IEEE operations (this file is
// compiled with -ffp-contract=off, so nothing else fuses), __ldg a plain load,
// and a warp's queue append one lane's append. The device compiler contracts
// some plain float expressions that this build does not, so the host results
// agree with the GPU's to the forms' tolerances, not bit for bit.
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

using std::isfinite;

namespace {
const uint3 threadIdx = {0u, 0u, 0u};
}
template <typename T>
static inline T __ldg(const T* p) {
  return *p;
}
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline long long __double_as_longlong(double d) {
  long long b;
  std::memcpy(&b, &d, sizeof(b));
  return b;
}
static inline float __int_as_float(int i) {
  float f;
  std::memcpy(&f, &i, sizeof(f));
  return f;
}
static inline int __double2hiint(double d) { return int(__double_as_longlong(d) >> 32); }
static inline int __double2loint(double d) { return int(unsigned(__double_as_longlong(d) & 0xffffffffLL)); }
// conversion rounded toward zero
static inline float __double2float_rz(double d) {
  float f = float(d);
  if (std::isinf(f) && std::isfinite(d)) return std::copysign(3.4028234663852886e38f, float(d));
  if (std::isfinite(d) && std::fabs(double(f)) > std::fabs(d)) f = std::nextafter(f, 0.f);
  return f;
}
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline int __ffs(unsigned x) { return __builtin_ffs(int(x)); }
static inline int __ffs(int x) { return __builtin_ffs(x); }
static inline unsigned __activemask() { return 1u; }
template <typename T>
static inline T __shfl_sync(unsigned, T v, int) {
  return v;
}
static inline unsigned atomicAdd(unsigned* p, unsigned v) {
  const unsigned old = *p;
  *p = old + v;
  return old;
}

#include "mixed_device.cuh"

using namespace mfgb;

namespace {

// search_kernel, screen_kernel, fix_kernel (two rounds), judge_kernel and
// repair_kernel of one condition set in the grid schedule's order (cold start)
template <int N, int K>
void cold_pipeline(const MixedArgs& a, const DevMixed& T, unsigned* qc) {
  qc[0] = qc[1] = 0u;  // zeroed by the search launch
  for (int64_t ch = 0; ch < a.n; ++ch) search_body<N, K, false>(a, T, ch);
  for (int64_t ch = 0; ch < a.n; ++ch) screen_body<N, K>(a, T, ch, qc + 1);
  for (unsigned i = 0; i < qc[1]; ++i) fix_body<N, K>(a, T, unsigned(a.ws_fixq[i]), 2);
  for (int64_t ch = 0; ch < a.n; ++ch) {
    if (a.judge_df) judge_df_body<N, K>(a, T, ch, qc, nullptr);
    else judge_body<N, K>(a, T, ch, qc, nullptr);
  }
  for (unsigned i = 0; i < qc[0]; ++i) judge_repair<N, K>(a, T, int64_t(a.ws_queue[i]));
}

// the warm start's order (launch_set): search from the predicted sets, judge
// (queueing channels with provably missing columns for the fix), fix (one
// round), the judge again on the fixed channels, repair
template <int N, int K>
void warm_pipeline(const MixedArgs& a, const DevMixed& T, unsigned* qc) {
  qc[0] = qc[1] = 0u;
  for (int64_t ch = 0; ch < a.n; ++ch) search_body<N, K, true>(a, T, ch);
  for (int64_t ch = 0; ch < a.n; ++ch) {
    if (a.judge_df) judge_df_body<N, K>(a, T, ch, qc, qc + 1);
    else judge_body<N, K>(a, T, ch, qc, qc + 1);
  }
  for (unsigned i = 0; i < qc[1]; ++i) fix_body<N, K>(a, T, unsigned(a.ws_fixq[i]), 1);
  for (unsigned i = 0; i < qc[1]; ++i) {
    const int64_t ch = int64_t(unsigned(a.ws_fixq[i]));
    if (a.judge_df) judge_df_body<N, K>(a, T, ch, qc, nullptr);
    else judge_body<N, K>(a, T, ch, qc, nullptr);
  }
  for (unsigned i = 0; i < qc[0]; ++i) judge_repair<N, K>(a, T, int64_t(a.ws_queue[i]));
}

}  // namespace

// Fits n channels of one condition set (mf_conditions layout, no pulse
// covariance, N = K = 10 or 8) with the cold-start pipeline, or, given
// predicted passive sets warm_mask[n] and amplitudes warm_amp[n][10] (N = K =
// 10), with the warm start's; judge_df: the judge in double-float FP32
// arithmetic (MF_PREC_FP32) instead of FP64. queues[2] returns the fix and
// repair queue lengths.
extern "C" int mixed_host(const mf_conditions* cond, const double* samples, const double* pederr, int64_t n,
                          int judge_df, int max_iter_nnls, double* amplitudes, double* chi2, uint16_t* active_mask,
                          uint8_t* status, int32_t* iters, unsigned* queues, const uint16_t* warm_mask,
                          const float* warm_amp) {
  const int N = cond->nsamples, K = cond->npulses;
  if (!((N == 10 && K == 10) || (N == 8 && K == 8)) || cond->has_fullpulsecov) return 1;
  if (warm_mask && N != 10) return 1;
  DevConditions* d = static_cast<DevConditions*>(std::calloc(1, sizeof(DevConditions)));
  if (!d) return 2;
  d->N = N;
  d->K = K;
  d->intime_col = -1;
  for (int k = 0; k < K; ++k) {
    d->bxs[k] = cond->bxs[k];
    if (d->intime_col < 0 && cond->bxs[k] == 0) d->intime_col = k;
  }
  for (int k = 0; k < K; ++k) {
    int fz = N;
    for (int i = 0; i < N; ++i) {
      d->P[k * N + i] = cond->pulse_matrix[k * N + i];
      if (fz == N && d->P[k * N + i] != 0.) fz = i;
    }
    d->fz[k] = int8_t(fz);
  }
  for (int i = 0; i < N * N; ++i) d->R[i] = cond->noise_cor[i];
  HostTables* h = new HostTables();
  const int rc = build_mixed_tables(*d, h);
  if (rc) {
    delete h;
    std::free(d);
    return 3;
  }
  // the device view of the tables (api.cu fill_dev_mixed), pointing at host memory
  DevMixed T;
  std::memset(&T, 0, sizeof(T));
  T.N = N;
  T.K = K;
  T.intime_col = d->intime_col;
  std::memcpy(T.W64, h->W64, sizeof(h->W64));
  std::memcpy(T.W32, h->W32, sizeof(h->W32));
  std::memcpy(T.W32lo, h->W32lo, sizeof(h->W32lo));
  std::memcpy(T.G64, h->G64, sizeof(h->G64));
  std::memcpy(T.H64, h->H64, sizeof(h->H64));
  std::memcpy(T.G32, h->G32, sizeof(h->G32));
  std::memcpy(T.G32lo, h->G32lo, sizeof(h->G32lo));
  std::memcpy(T.P32, h->P32, sizeof(h->P32));
  std::memcpy(T.P32lo, h->P32lo, sizeof(h->P32lo));
  std::memcpy(T.H32, h->H32, sizeof(h->H32));
  for (int k = 0; k < K; ++k) {
    T.gnorm32[k] = float(std::sqrt(h->gnorm2[k]));
    T.gfz[k] = int8_t(h->gfz[k]);
  }
  T.zero_row = h->offset[size_t(1) << K];
  T.offset = h->offset.data();
  T.pinv64 = h->pinv64.data();
  T.pinv32 = h->pinv32.data();
  T.pinv32lo = h->pinv32lo.data();
  T.pinv2 = h->pinv2.data();
  T.g2 = h->pinv2.data() + h->g2_off;
  // G in its own (16-byte aligned) array, as the device copy the judge reads
  // with 16-byte loads
  std::vector<double> g64(h->G64, h->G64 + N * K);
  T.g64 = g64.data();

  std::vector<uint16_t> ws_mask(n), ws_count(n), ws_add(n);
  std::vector<float> ws_x(size_t(n) * K);
  std::vector<int> ws_queue(n), ws_fixq(n);
  unsigned qc[2] = {0u, 0u};
  MixedArgs* a = static_cast<MixedArgs*>(std::calloc(1, sizeof(MixedArgs)));
  if (!a) {
    delete h;
    std::free(d);
    return 2;
  }
  a->tab[0] = T;
  a->n_ctypes = 1;
  a->skip_set = -1;
  a->warm_set = -1;
  a->n = n;
  a->sample_stride = N;
  a->amp_stride = K;
  a->max_iter32 = 12;  // mf_fit's settings of the mixed and FP32 precisions
  a->max_iter64 = max_iter_nnls > 0 ? max_iter_nnls : 1;
  a->tol32 = 1e-5f;
  a->eps = 1e-11;
  a->eps32 = float(1e-11);
  a->samples = samples;
  a->pederr = pederr;
  a->amplitudes = amplitudes;
  a->chi2 = chi2;
  a->active_mask = active_mask;
  a->status = status;
  a->iters = iters;
  a->ws_mask = ws_mask.data();
  a->ws_count = ws_count.data();
  a->ws_x = ws_x.data();
  a->ws_queue = ws_queue.data();
  a->ws_fixq = ws_fixq.data();
  a->ws_add = ws_add.data();
  a->ws_qcount = qc;
  a->sms = 1;
  a->list_identity = 1;
  a->judge_df = judge_df ? 1 : 0;
  if (warm_mask) {
    a->warm_mask = warm_mask;
    a->warm_amp = warm_amp;
    a->warm_stride = 10;
    a->warm_set = 0;
    warm_pipeline<10, 10>(*a, a->tab[0], qc);
  } else if (N == 10) {
    cold_pipeline<10, 10>(*a, a->tab[0], qc);
  } else {
    cold_pipeline<8, 8>(*a, a->tab[0], qc);
  }
  queues[0] = qc[1];
  queues[1] = qc[0];
  std::free(a);
  delete h;
  std::free(d);
  return 0;
}
