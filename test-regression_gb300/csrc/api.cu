// C ABI of the engine (include/multifit_gb300.h).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "mf_internal.h"
#include "mlp.h"
#include "mlp_state.h"

namespace mfgb {

static thread_local char g_last_error[256] = "";

void set_last_error(const char* what, cudaError_t e) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%d)", what, cudaGetErrorString(e), int(e));
}

int make_dev_conditions(const mf_conditions& c, DevConditions* d) {
  const int N = c.nsamples, K = c.npulses;
  if (N < 1 || N > KMAX || K < 1 || K > KMAX) return MF_EINVAL;
  std::memset(d, 0, sizeof(*d));
  d->N = N;
  d->K = K;
  d->intime_col = -1;
  for (int k = 0; k < K; ++k) {
    d->bxs[k] = c.bxs[k];
    if (d->intime_col < 0 && c.bxs[k] == 0) d->intime_col = k;
  }
  for (int k = 0; k < K; ++k) {
    int fz = N;
    for (int i = 0; i < N; ++i) {
      const double v = c.pulse_matrix[k * N + i];
      d->P[k * N + i] = v;
      if (fz == N && v != 0.) fz = i;
    }
    d->fz[k] = int8_t(fz);
  }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) d->R[j * N + i] = c.noise_cor[j * N + i];
  d->has_fpc = c.has_fullpulsecov ? 1 : 0;
  if (d->has_fpc) {
    const int NF = N + 9;
    for (int k = 0; k < K; ++k)  // the pulse-covariance block rule needs bx in [-N+1, 6]
      if (c.bxs[k] < -(N - 1) || c.bxs[k] > 6) return MF_EINVAL;
    std::memcpy(d->fpc, c.fullpulsecov, sizeof(double) * NF * NF);
  }
  return MF_OK;
}

}  // namespace mfgb

using namespace mfgb;

// The launch arguments a captured persistent-schedule graph was built from;
// a call with byte-identical arguments replays the graph.
struct GraphKey {
  MixedArgs m;
  MlpInferArgs ia;
  int warm, block, lanes;
};

// The mixed form's per-fit device workspace: the search -> judge hand-off,
// the fix and repair queues, the persistent schedule's lists and counters,
// and the warm start's predictions. Lane 0 is the context's own workspace;
// mf_fit_host runs alternate chunks on lane 1 (second stream) as well.
struct Lane {
  uint16_t* mask = nullptr;
  uint16_t* count = nullptr;
  float* x = nullptr;
  int* queue = nullptr;
  int* fixq = nullptr;
  uint16_t* add = nullptr;
  unsigned* qcount = nullptr;
  int* list = nullptr;
  unsigned* sched = nullptr;
  uint16_t* warm_mask = nullptr;
  float* warm_amp = nullptr;
};

struct mf_context {
  int device = 0;
  DevConditions cond[MF_MAX_CTYPES];
  int cond_set[MF_MAX_CTYPES] = {0, 0};
  // mixed / warm-start tables per condition set (built by mf_set_conditions)
  HostTables tab[MF_MAX_CTYPES];
  int tab_ok[MF_MAX_CTYPES] = {0, 0};
  int* d_offset[MF_MAX_CTYPES] = {nullptr, nullptr};
  double* d_pinv64[MF_MAX_CTYPES] = {nullptr, nullptr};
  float* d_pinv32[MF_MAX_CTYPES] = {nullptr, nullptr};
  float* d_pinv32lo[MF_MAX_CTYPES] = {nullptr, nullptr};
  float* d_pinv2[MF_MAX_CTYPES] = {nullptr, nullptr};
  double* d_g64[MF_MAX_CTYPES] = {nullptr, nullptr};
  MlpState mlp;
  int sms = 152;
  // mixed-form hand-off workspace (MIXED_CHUNK channels), allocated with the tables
  uint16_t* ws_mask = nullptr;
  uint16_t* ws_count = nullptr;
  float* ws_x = nullptr;
  int* ws_queue = nullptr;
  int* ws_fixq = nullptr;
  uint16_t* ws_add = nullptr;
  unsigned* ws_qcount = nullptr;
  // persistent schedule: per-set channel lists and counters; tuned launch shape
  int* ws_list = nullptr;
  unsigned* ws_sched = nullptr;
  int tuned_block = 0;  // mf_autotune result (0: not tuned, use 128)
  int tuned_lanes = 0;  // lanes per channel of the FP32 search (0: not tuned, use 1)
  // CUDA graph of the last persistent-schedule fit (captured on cap_stream)
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  GraphKey graph_key;
  // staging area for mf_fit_host
  int64_t cap = 0;
  int cap_ss = 0, cap_as = 0;
  double* d_samples = nullptr;
  double* d_pederr = nullptr;
  uint8_t* d_ctype = nullptr;
  double* d_amp = nullptr;
  double* d_chi2 = nullptr;
  double* d_intime = nullptr;
  double* d_errors = nullptr;
  uint16_t* d_mask = nullptr;
  uint8_t* d_status = nullptr;
  int32_t* d_iters = nullptr;
  cudaStream_t stream = nullptr;
  // mf_fit_host pipeline: copy-in and copy-out streams, per-chunk events, and
  // a second compute stream with its own workspace (lane 1, allocated on
  // first use)
  cudaStream_t h2d_stream = nullptr, d2h_stream = nullptr;
  cudaStream_t stream2 = nullptr;
  Lane lane1;
  cudaEvent_t fork = nullptr;
  static constexpr int kHostChunks = 64;
  cudaEvent_t in_done[kHostChunks] = {}, fit_done[kHostChunks] = {};
  LaunchTimer timer;  // per-kernel launch timing (mf_profile), off by default
  std::mutex mu;
};

namespace {

int check_options(const mf_options* o) {
  if (!o) return MF_EINVAL;
  if (o->max_iter_nnls < 0 || o->max_iter_outer < 0) return MF_EINVAL;
  if (!(o->dchi2_tol >= 0) || !(o->nnls_eps >= 0)) return MF_EINVAL;
  if (o->precision != MF_PREC_FP64 && o->precision != MF_PREC_MIXED && o->precision != MF_PREC_FP32)
    return MF_EINVAL;
  if (o->schedule != MF_SCHED_GRID && o->schedule != MF_SCHED_PERSISTENT) return MF_EINVAL;
  if (o->warm_start != MF_WARM_NONE && o->warm_start != MF_WARM_MLP) return MF_EINVAL;
  if (o->nnls_start != MF_START_REFERENCE && o->nnls_start != MF_START_SUPPORT) return MF_EINVAL;
  if (o->block_size < 0 || o->block_size > 1024 || (o->block_size % 32)) return MF_EINVAL;
  if (o->blocks_per_sm < 0) return MF_EINVAL;
  const int cpw = o->channels_per_warp;
  if (cpw != 0 && cpw != 1 && cpw != 2 && cpw != 4 && cpw != 8 && cpw != 32) return MF_EINVAL;
  if (o->schedule == MF_SCHED_PERSISTENT && o->block_size > 512) return MF_EINVAL;
  // the grid schedule's kernels are compiled for at most 128 threads a block
  if (o->schedule == MF_SCHED_GRID && o->block_size > 128) {
    std::snprintf(g_last_error, sizeof(g_last_error),
                  "block_size %d: the grid schedule takes at most 128 threads a block", o->block_size);
    return MF_EINVAL;
  }
  return MF_OK;
}

int fill_args(mf_context* ctx, const mf_batch* b, const mf_options* o, FitArgs* a) {
  if (!ctx || !b) return MF_EINVAL;
  int rc = check_options(o);
  if (rc) return rc;
  if (b->n < 0 || (b->n > 0 && (!b->samples || !b->pederr || !b->amplitudes || !b->chi2))) return MF_EINVAL;
  int nct = 0;
  for (int t = 0; t < MF_MAX_CTYPES; ++t)
    if (ctx->cond_set[t]) nct = t + 1;
  if (nct == 0 || !ctx->cond_set[0]) return MF_EINVAL;
  if (!b->ctype) nct = 1;
  for (int t = 0; t < nct; ++t) {
    if (!ctx->cond_set[t]) return MF_EINVAL;
    if (b->sample_stride < ctx->cond[t].N || b->amp_stride < ctx->cond[t].K) return MF_EINVAL;
    a->cond[t] = ctx->cond[t];
  }
  a->n_ctypes = nct;
  a->opt.max_iter_nnls = o->max_iter_nnls;
  a->opt.max_iter_outer = o->max_iter_outer;
  a->opt.dchi2_tol = o->dchi2_tol;
  a->opt.nnls_eps = o->nnls_eps;
  a->opt.nnls_start = o->nnls_start;
  a->opt.compute_errors = o->compute_errors;
  a->n = b->n;
  a->sample_stride = b->sample_stride;
  a->amp_stride = b->amp_stride;
  a->samples = b->samples;
  a->pederr = b->pederr;
  a->ctype = b->ctype;
  a->amplitudes = b->amplitudes;
  a->chi2 = b->chi2;
  a->intime = b->intime;
  a->errors = b->errors;
  a->active_mask = b->active_mask;
  a->status = b->status;
  a->iters = b->iters;
  a->flops = nullptr;
  a->seeded = 0;
  a->sms = ctx->sms;
  return MF_OK;
}

void fill_dev_mixed(const mf_context* c, int t, DevMixed* m);

int dispatch_mixed(mf_context* c, const FitArgs& a, const mf_options* o, cudaStream_t s, bool allow_graph,
                   int lane) {
  if (o->compute_errors) return MF_EUNSUPPORTED;
  const bool persistent = o->schedule == MF_SCHED_PERSISTENT;
  const int block = o->block_size ? o->block_size : (persistent && c->tuned_block ? c->tuned_block : 128);
  const int lanes = o->channels_per_warp ? 32 / o->channels_per_warp : (c->tuned_lanes ? c->tuned_lanes : 1);
  const bool warm = o->warm_start == MF_WARM_MLP;
  if (warm && (!c->mlp.trained || !c->tab_ok[c->mlp.set] || c->tab[c->mlp.set].N != 10)) return MF_ENOTRAINED;
  MixedArgs m;
  std::memset(&m, 0, sizeof(m));
  for (int t = 0; t < a.n_ctypes; ++t) {
    if (!c->tab_ok[t]) return MF_EUNSUPPORTED;
    fill_dev_mixed(c, t, &m.tab[t]);
  }
  m.n_ctypes = a.n_ctypes;
  m.skip_set = -1;
  m.warm_set = -1;
  m.n = a.n;
  m.sample_stride = a.sample_stride;
  m.amp_stride = a.amp_stride;
  // outer iterations of a cold FP32 search (the warm search has its own cap):
  // past 12 a channel is left to the screen, the fix and the judge (10M cold
  // ECAL channels: 8.84 ms per step with 30, 8.72 with 12, 8.78 with 8 and
  // 15.8 with 6, when the repair queue grew tenfold)
  m.max_iter32 = 12;
  m.max_iter64 = o->max_iter_nnls > 0 ? o->max_iter_nnls : 1;
  m.tol32 = 1e-5f;
  m.eps = o->nnls_eps;
  m.eps32 = float(o->nnls_eps);
  m.samples = a.samples;
  m.pederr = a.pederr;
  m.ctype = a.ctype;
  m.amplitudes = a.amplitudes;
  m.chi2 = a.chi2;
  m.intime = a.intime;
  m.active_mask = a.active_mask;
  m.status = a.status;
  m.iters = a.iters;
  m.flops = a.flops;
  m.ws_mask = c->ws_mask;
  m.ws_count = c->ws_count;
  m.ws_x = c->ws_x;
  m.ws_queue = c->ws_queue;
  m.ws_fixq = c->ws_fixq;
  m.ws_add = c->ws_add;
  m.ws_qcount = c->ws_qcount;
  m.sms = c->sms;
  m.ws_list = c->ws_list;
  m.ws_sched = c->ws_sched;
  uint16_t* warm_mask = c->mlp.warm_mask;
  float* warm_amp = c->mlp.warm_amp;
  if (lane == 1) {
    const Lane& L = c->lane1;
    m.ws_mask = L.mask;
    m.ws_count = L.count;
    m.ws_x = L.x;
    m.ws_queue = L.queue;
    m.ws_fixq = L.fixq;
    m.ws_add = L.add;
    m.ws_qcount = L.qcount;
    m.ws_list = L.list;
    m.ws_sched = L.sched;
    warm_mask = L.warm_mask;
    warm_amp = L.warm_amp;
  }
  m.blocks_per_sm = o->blocks_per_sm;
  m.list_identity = a.ctype == nullptr ? 1 : 0;
  m.judge_df = o->precision == MF_PREC_FP32 ? 1 : 0;
  if (!m.ws_mask || !m.ws_list) return MF_ENOMEM;
  MlpInferArgs ia;
  std::memset(&ia, 0, sizeof(ia));
  if (warm) {
    fill_infer_args(c->mlp, c->tab[c->mlp.set], 0, &ia);
    ia.sample_stride = a.sample_stride;
    ia.warm_mask = warm_mask;
    ia.warm_amp = warm_amp;
    ia.warm_stride = 10;
  }
  const int64_t cap = warm && MlpState::kChunk < MIXED_CHUNK ? MlpState::kChunk : MIXED_CHUNK;
  // every launch of the fit, chunk by chunk, on stream st
  auto enqueue = [&](cudaStream_t st, LaunchTimer* tm) -> cudaError_t {
  // chunks of equal size, at most cap each
  const int64_t nch = a.n > cap ? (a.n + cap - 1) / cap : 1;
  const int64_t even = a.n > 0 ? (a.n + nch - 1) / nch : 1;
  for (int64_t off = 0; off < a.n; off += even) {
    const int64_t cnt = a.n - off < even ? a.n - off : even;
    MixedArgs mc = m;
    mc.n = cnt;
    mc.samples = a.samples + off * a.sample_stride;
    mc.pederr = a.pederr + off;
    mc.ctype = a.ctype ? a.ctype + off : nullptr;
    mc.amplitudes = a.amplitudes + off * a.amp_stride;
    mc.chi2 = a.chi2 + off;
    mc.intime = a.intime ? a.intime + off : nullptr;
    mc.active_mask = a.active_mask ? a.active_mask + off : nullptr;
    mc.status = a.status ? a.status + off : nullptr;
    mc.iters = a.iters ? a.iters + off : nullptr;
    mc.flops = a.flops ? a.flops + off : nullptr;
    cudaError_t e = cudaSuccess;
    if (warm) {
      // learned warm start: predictions of this chunk into the network's workspace
      MlpInferArgs ic = ia;
      ic.n = cnt;
      ic.samples = mc.samples;
      ic.pederr = mc.pederr;
      ic.ctype = mc.ctype;
      mc.warm_mask = warm_mask;
      mc.warm_amp = warm_amp;
      mc.warm_stride = 10;
      mc.warm_set = c->mlp.set;
      if (tm) tm->mark(MF_K_MLP_INFER, st);
      e = launch_mlp_infer(ic, c->sms, st);
    }
    if (e == cudaSuccess) {
      e = persistent ? launch_fit_mixed_persistent(mc, block, lanes, st, tm)
                     : launch_fit_mixed(mc, o->block_size, st, tm);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
  };
  cudaError_t e = cudaSuccess;
  if (!persistent || c->timer.ev || !allow_graph) {
    // grid schedule, per-launch timing requested, or a caller that varies the
    // arguments every call (the chunks of mf_fit_host): launch directly
    e = enqueue(s, &c->timer);
  } else {
    // persistent schedule: replay the CUDA graph of this exact launch sequence,
    // capturing (and instantiating) it first when the arguments changed
    GraphKey key;
    std::memset(&key, 0, sizeof(key));
    key.m = m;
    key.ia = ia;
    key.warm = warm;
    key.block = block;
    key.lanes = lanes;
    if (!c->graph_exec || std::memcmp(&key, &c->graph_key, sizeof(key)) != 0) {
      if (!c->cap_stream) e = cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking);
      cudaGraph_t g = nullptr;
      if (e == cudaSuccess) e = cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const cudaError_t le = enqueue(c->cap_stream, nullptr);
        e = cudaStreamEndCapture(c->cap_stream, &g);
        if (le != cudaSuccess) e = le;
      }
      cudaGraphExec_t x = nullptr;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e == cudaSuccess) {
        if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
        c->graph_exec = x;
        c->graph_key = key;
      }
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(c->graph_exec, s);
  }
  if (e != cudaSuccess) {
    set_last_error("mixed fit launch", e);
    return MF_ECUDA;
  }
  return MF_OK;
}

// The mixed and FP32 precisions fit a batch through the passive-set tables
// alone when every condition set it uses has them, none has a pulse
// covariance and no errors are asked for. Otherwise they take the per-channel
// form: with the amplitudes at zero, the reference's first outer iteration
// (PulseChiSqSNNLS.cpp:149-166) fits with the covariance pederr^2 samplecor --
// exactly the tables' problem -- so that iteration (the costly one: its FNNLS
// starts from an empty passive set) runs through the tables, and the FP64 fit
// continues the outer loop from it: the covariance built from those
// amplitudes (with the pulse covariance), FNNLS from their support, the
// stopping rule against their chi2, then the MINOS-like refits. The result
// follows the FP64 trajectory from the second iteration on. Sets without
// tables (shapes other than N = K = 10 or 8) run the whole loop in FP64.
int dispatch_per_channel(mf_context* c, const FitArgs& a, const mf_options* o, cudaStream_t s, bool instrumented,
                         bool allow_graph, int lane) {
  bool tables = true;
  for (int t = 0; t < a.n_ctypes; ++t)
    if (!c->tab_ok[t]) tables = false;
  FitArgs a64 = a;
  a64.opt.nnls_start = MF_START_SUPPORT;
  a64.opt.max_iter_nnls = o->max_iter_nnls > 0 ? o->max_iter_nnls : 1;
  if (tables) {
    mf_options first = *o;
    first.compute_errors = 0;
    const int rc = dispatch_mixed(c, a, &first, s, allow_graph, lane);
    if (rc) return rc;
    a64.seeded = 1;
  }
  const int block = o->block_size && o->block_size <= 128 ? o->block_size : 128;
  const cudaError_t e = launch_fit_fp64(a64, block, s, instrumented, &c->timer);
  if (e != cudaSuccess) {
    set_last_error("per-channel fit launch", e);
    return MF_ECUDA;
  }
  return MF_OK;
}

bool per_channel_form(const mf_context* c, const FitArgs& a, const mf_options* o) {
  if (o->compute_errors) return true;
  for (int t = 0; t < a.n_ctypes; ++t)
    if (!c->tab_ok[t] || c->cond[t].has_fpc) return true;
  return false;
}

int dispatch_form(mf_context* c, const FitArgs& a, const mf_options* o, cudaStream_t s, bool instrumented,
                  bool allow_graph, int lane) {
  if ((o->precision == MF_PREC_MIXED || o->precision == MF_PREC_FP32) && per_channel_form(c, a, o))
    return dispatch_per_channel(c, a, o, s, instrumented, allow_graph, lane);
  if (o->precision == MF_PREC_MIXED || o->precision == MF_PREC_FP32)
    return dispatch_mixed(c, a, o, s, allow_graph, lane);
  if (o->precision != MF_PREC_FP64 || o->schedule != MF_SCHED_GRID || o->warm_start != MF_WARM_NONE)
    return MF_EUNSUPPORTED;
  cudaError_t e = launch_fit_fp64(a, o->block_size, s, instrumented, &c->timer);
  if (e != cudaSuccess) {
    set_last_error("fit_fp64 launch", e);
    return MF_ECUDA;
  }
  return MF_OK;
}

int dispatch(mf_context* c, const FitArgs& a, const mf_options* o, cudaStream_t s, bool instrumented,
             bool allow_graph = true, int lane = 0) {
  const int rc = dispatch_form(c, a, o, s, instrumented, allow_graph, lane);
  c->timer.mark(-1, s);  // end of this fit's launches
  return rc;
}

void destroy_timer(LaunchTimer& t) {
  if (!t.ev) return;
  for (int i = 0; i < LaunchTimer::kEvents; ++i) cudaEventDestroy(t.ev[i]);
  delete[] t.ev;
  t.ev = nullptr;
  t.used = 0;
  t.overflow = false;
}

void free_lane(Lane& L) {
  void* ps[] = {L.mask, L.count, L.x, L.queue, L.fixq, L.add, L.qcount, L.list, L.sched, L.warm_mask, L.warm_amp};
  for (void* p : ps) cudaFree(p);
  L = Lane();
}

// Lane 1 and the second compute stream of mf_fit_host (~1.7 GB with the
// warm-start predictions), once.
int grow_lane1(mf_context* c) {
  if (c->lane1.mask) return MF_OK;
  Lane& L = c->lane1;
  cudaError_t e = cudaMalloc(&L.mask, sizeof(uint16_t) * MIXED_CHUNK);
  if (e == cudaSuccess) e = cudaMalloc(&L.count, sizeof(uint16_t) * MIXED_CHUNK);
  if (e == cudaSuccess) e = cudaMalloc(&L.x, sizeof(float) * MIXED_CHUNK * KMAX);
  if (e == cudaSuccess) e = cudaMalloc(&L.queue, sizeof(int) * MIXED_CHUNK);
  if (e == cudaSuccess) e = cudaMalloc(&L.fixq, sizeof(int) * MIXED_CHUNK);
  if (e == cudaSuccess) e = cudaMalloc(&L.add, sizeof(uint16_t) * MIXED_CHUNK);
  if (e == cudaSuccess) e = cudaMalloc(&L.qcount, 2 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&L.list, sizeof(int) * MIXED_CHUNK * MF_MAX_CTYPES);
  if (e == cudaSuccess) e = cudaMalloc(&L.sched, sizeof(unsigned) * SCHED_WORDS);
  if (e == cudaSuccess) e = cudaMalloc(&L.warm_mask, sizeof(uint16_t) * MlpState::kChunk);
  if (e == cudaSuccess) e = cudaMalloc(&L.warm_amp, sizeof(float) * MlpState::kChunk * 10);
  if (e == cudaSuccess && !c->stream2) e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking);
  if (e == cudaSuccess && !c->fork) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    set_last_error("mf_fit_host: second lane", e);
    free_lane(L);
    return MF_ENOMEM;
  }
  return MF_OK;
}

void free_staging(mf_context* c) {
  cudaFree(c->d_samples);
  cudaFree(c->d_pederr);
  cudaFree(c->d_ctype);
  cudaFree(c->d_amp);
  cudaFree(c->d_chi2);
  cudaFree(c->d_intime);
  cudaFree(c->d_errors);
  cudaFree(c->d_mask);
  cudaFree(c->d_status);
  cudaFree(c->d_iters);
  c->d_samples = nullptr;
  c->d_pederr = nullptr;
  c->d_ctype = nullptr;
  c->d_amp = c->d_chi2 = c->d_intime = c->d_errors = nullptr;
  c->d_mask = nullptr;
  c->d_status = nullptr;
  c->d_iters = nullptr;
  c->cap = 0;
}

void free_tables(mf_context* c, int t) {
  cudaFree(c->d_offset[t]);
  cudaFree(c->d_pinv64[t]);
  cudaFree(c->d_pinv32[t]);
  cudaFree(c->d_pinv32lo[t]);
  cudaFree(c->d_pinv2[t]);
  cudaFree(c->d_g64[t]);
  c->d_g64[t] = nullptr;
  c->d_pinv32lo[t] = nullptr;
  c->d_pinv2[t] = nullptr;
  c->d_offset[t] = nullptr;
  c->d_pinv64[t] = nullptr;
  c->d_pinv32[t] = nullptr;
  c->tab_ok[t] = 0;
}

// Builds the mixed-form tables of set t and uploads them. The tables depend on
// the pulse matrix and samplecor only, so a set with a pulse covariance has
// them too (they serve its first outer iteration). A set they cannot serve
// (K > N, a shape without a build, or a non-positive-definite samplecor)
// keeps tab_ok = 0; the mixed precision then fits it in FP64 throughout.
int upload_tables(mf_context* c, int t) {
  free_tables(c, t);
  const DevConditions& d = c->cond[t];
  const bool shape_ok = (d.N == 10 && d.K == 10) || (d.N == 8 && d.K == 8);
  if (!shape_ok) return MF_OK;
  HostTables& h = c->tab[t];
  if (build_mixed_tables(d, &h) != MF_OK) return MF_OK;
  cudaError_t e = cudaSetDevice(c->device);
  const size_t no = h.offset.size(), np = h.pinv64.size();
  if (e == cudaSuccess) e = cudaMalloc(&c->d_offset[t], sizeof(int) * no);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_pinv64[t], sizeof(double) * np);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_pinv32[t], sizeof(float) * np);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_pinv32lo[t], sizeof(float) * np);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_pinv2[t], sizeof(float) * h.pinv2.size());
  if (e == cudaSuccess) e = cudaMemcpy(c->d_offset[t], h.offset.data(), sizeof(int) * no, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c->d_pinv64[t], h.pinv64.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c->d_pinv32[t], h.pinv32.data(), sizeof(float) * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->d_pinv32lo[t], h.pinv32lo.data(), sizeof(float) * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->d_pinv2[t], h.pinv2.data(), sizeof(float) * h.pinv2.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_g64[t], sizeof(double) * size_t(d.N) * d.K);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->d_g64[t], h.G64, sizeof(double) * size_t(d.N) * d.K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !c->ws_mask) {
    e = cudaMalloc(&c->ws_mask, sizeof(uint16_t) * MIXED_CHUNK);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_count, sizeof(uint16_t) * MIXED_CHUNK);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_x, sizeof(float) * MIXED_CHUNK * KMAX);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_queue, sizeof(int) * MIXED_CHUNK);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_fixq, sizeof(int) * MIXED_CHUNK);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_add, sizeof(uint16_t) * MIXED_CHUNK);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_qcount, 2 * sizeof(unsigned));  // repair and fix queues
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_list, sizeof(int) * MIXED_CHUNK * MF_MAX_CTYPES);
    if (e == cudaSuccess) e = cudaMalloc(&c->ws_sched, sizeof(unsigned) * SCHED_WORDS);
  }
  if (e != cudaSuccess) {
    set_last_error("table upload", e);
    free_tables(c, t);
    return MF_ECUDA;
  }
  c->tab_ok[t] = 1;
  return MF_OK;
}

void fill_dev_mixed(const mf_context* c, int t, DevMixed* m) {
  const HostTables& h = c->tab[t];
  const int N = h.N, K = h.K;
  std::memset(m, 0, sizeof(*m));
  m->N = N;
  m->K = K;
  m->intime_col = c->cond[t].intime_col;
  std::memcpy(m->W64, h.W64, sizeof(h.W64));
  std::memcpy(m->W32, h.W32, sizeof(h.W32));
  std::memcpy(m->W32lo, h.W32lo, sizeof(h.W32lo));
  std::memcpy(m->G64, h.G64, sizeof(h.G64));
  std::memcpy(m->H64, h.H64, sizeof(h.H64));
  std::memcpy(m->G32, h.G32, sizeof(h.G32));
  std::memcpy(m->G32lo, h.G32lo, sizeof(h.G32lo));
  std::memcpy(m->P32, h.P32, sizeof(h.P32));
  std::memcpy(m->P32lo, h.P32lo, sizeof(h.P32lo));
  std::memcpy(m->H32, h.H32, sizeof(h.H32));
  for (int k = 0; k < K; ++k) {
    m->gnorm32[k] = float(std::sqrt(h.gnorm2[k]));
    m->gfz[k] = int8_t(h.gfz[k]);
  }
  m->zero_row = h.offset[size_t(1) << K];
  m->offset = c->d_offset[t];
  m->pinv64 = c->d_pinv64[t];
  m->pinv32 = c->d_pinv32[t];
  m->pinv32lo = c->d_pinv32lo[t];
  m->pinv2 = c->d_pinv2[t];
  m->g2 = c->d_pinv2[t] + h.g2_off;
  m->g64 = c->d_g64[t];
}

int grow_staging(mf_context* c, int64_t n, int ss, int as) {
  if (n <= c->cap && ss <= c->cap_ss && as <= c->cap_as) return MF_OK;
  free_staging(c);
  cudaError_t e = cudaSuccess;
  auto al = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 1);
  };
  al((void**)&c->d_samples, sizeof(double) * n * ss);
  al((void**)&c->d_pederr, sizeof(double) * n);
  al((void**)&c->d_ctype, n);
  al((void**)&c->d_amp, sizeof(double) * n * as);
  al((void**)&c->d_chi2, sizeof(double) * n);
  al((void**)&c->d_intime, sizeof(double) * n);
  al((void**)&c->d_errors, sizeof(double) * n);
  al((void**)&c->d_mask, sizeof(uint16_t) * n);
  al((void**)&c->d_status, n);
  al((void**)&c->d_iters, sizeof(int32_t) * n);
  if (e != cudaSuccess) {
    set_last_error("staging cudaMalloc", e);
    free_staging(c);
    return MF_ENOMEM;
  }
  c->cap = n;
  c->cap_ss = ss;
  c->cap_as = as;
  return MF_OK;
}

}  // namespace

extern "C" {

int mf_abi_version(void) { return MF_ABI_VERSION; }

const char* mf_rc_string(int rc) {
  switch (rc) {
    case MF_OK: return "ok";
    case MF_EINVAL: return "invalid argument";
    case MF_ECUDA: return "CUDA error";
    case MF_ETIMEOUT: return "device-side wait timed out";
    case MF_ENOMEM: return "out of device memory";
    case MF_EUNSUPPORTED: return "unsupported option combination";
    case MF_ENOTRAINED: return "MLP weights not set";
    default: return "unknown error";
  }
}

const char* mf_last_error(void) { return g_last_error; }

void mf_default_options(mf_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->max_iter_nnls = 10;
  o->max_iter_outer = 50;
  o->dchi2_tol = 1e-3;
  o->nnls_eps = 1e-11;
  o->nnls_start = MF_START_REFERENCE;
  o->precision = MF_PREC_FP64;
  o->schedule = MF_SCHED_GRID;
  o->warm_start = MF_WARM_NONE;
  o->compute_errors = 0;
  o->block_size = 0;
  o->blocks_per_sm = 0;
}

int mf_create(mf_context** out, int device) {
  if (!out) return MF_EINVAL;
  *out = nullptr;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    set_last_error("cudaSetDevice", e);
    return MF_ECUDA;
  }
  mf_context* c = new (std::nothrow) mf_context();
  if (!c) return MF_ENOMEM;
  c->device = device;
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    set_last_error("cudaStreamCreate", e);
    delete c;
    return MF_ECUDA;
  }
  *out = c;
  return MF_OK;
}

void mf_destroy(mf_context* c) {
  if (!c) return;
  free_staging(c);
  for (int t = 0; t < MF_MAX_CTYPES; ++t) free_tables(c, t);
  mlp_free(c->mlp);
  cudaFree(c->ws_mask);
  cudaFree(c->ws_count);
  cudaFree(c->ws_x);
  cudaFree(c->ws_queue);
  cudaFree(c->ws_fixq);
  cudaFree(c->ws_add);
  cudaFree(c->ws_qcount);
  cudaFree(c->ws_list);
  cudaFree(c->ws_sched);
  free_lane(c->lane1);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->fork) cudaEventDestroy(c->fork);
  destroy_timer(c->timer);
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
  for (int i = 0; i < mf_context::kHostChunks; ++i) {
    if (c->in_done[i]) cudaEventDestroy(c->in_done[i]);
    if (c->fit_done[i]) cudaEventDestroy(c->fit_done[i]);
  }
  if (c->h2d_stream) cudaStreamDestroy(c->h2d_stream);
  if (c->d2h_stream) cudaStreamDestroy(c->d2h_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int mf_autotune(mf_context* c, const mf_batch* b, const mf_options* o, mf_tune_point* points, int max_points,
                int* n_points) {
  if (n_points) *n_points = 0;
  FitArgs a;
  int rc = fill_args(c, b, o, &a);
  if (rc) return rc;
  if (o->precision != MF_PREC_MIXED && o->precision != MF_PREC_FP32) return MF_EUNSUPPORTED;
  if (b->n == 0 || max_points < 0 || (max_points > 0 && !points)) return MF_EINVAL;
  static const int blocks[] = {64, 128, 256, 512};
  static const int cpws[] = {32, 8, 4, 2, 1};
  cudaStream_t s = c->stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  int best_block = 0, best_cpw = 0, n = 0;
  double best = 0.;
  for (int bi = 0; bi < 4 && e == cudaSuccess && rc == MF_OK; ++bi) {
    for (int ci = 0; ci < 5 && e == cudaSuccess && rc == MF_OK; ++ci) {
      mf_options t = *o;
      t.schedule = MF_SCHED_PERSISTENT;
      t.block_size = blocks[bi];
      t.channels_per_warp = cpws[ci];
      double ms_best = 0.;
      for (int rep = 0; rep < 4 && rc == MF_OK && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) rc = dispatch(c, a, &t, s, false);
        if (rc == MF_OK && e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (rc == MF_OK && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (rc == MF_OK && e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (rep == 1 || ms < ms_best)) ms_best = ms;  // rep 0 is the warm-up (and graph capture)
      }
      if (rc != MF_OK || e != cudaSuccess) break;
      if (n < max_points) points[n] = mf_tune_point{blocks[bi], cpws[ci], ms_best};
      ++n;
      if (best_block == 0 || ms_best < best) {
        best = ms_best;
        best_block = blocks[bi];
        best_cpw = cpws[ci];
      }
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc != MF_OK) return rc;
  if (e != cudaSuccess) {
    set_last_error("mf_autotune", e);
    return MF_ECUDA;
  }
  c->tuned_block = best_block;
  c->tuned_lanes = 32 / best_cpw;
  if (n_points) *n_points = n < max_points ? n : max_points;
  return MF_OK;
}

int mf_profile(mf_context* c, int enable) {
  if (!c) return MF_EINVAL;
  std::lock_guard<std::mutex> g(c->mu);
  destroy_timer(c->timer);
  if (!enable) return MF_OK;
  c->timer.ev = new (std::nothrow) cudaEvent_t[LaunchTimer::kEvents];
  if (!c->timer.ev) return MF_ENOMEM;
  cudaError_t e = cudaSetDevice(c->device);
  int made = 0;
  for (; made < LaunchTimer::kEvents && e == cudaSuccess; ++made) e = cudaEventCreate(&c->timer.ev[made]);
  if (e != cudaSuccess) {
    for (int i = 0; i + 1 < made; ++i) cudaEventDestroy(c->timer.ev[i]);
    delete[] c->timer.ev;
    c->timer.ev = nullptr;
    set_last_error("mf_profile: cudaEventCreate", e);
    return MF_ECUDA;
  }
  return MF_OK;
}

int mf_profile_read(mf_context* c, int32_t* launches, double* total_ms) {
  if (!c || !launches || !total_ms) return MF_EINVAL;
  std::lock_guard<std::mutex> g(c->mu);
  for (int k = 0; k < MF_K_COUNT; ++k) {
    launches[k] = 0;
    total_ms[k] = 0.;
  }
  LaunchTimer& t = c->timer;
  if (!t.ev) return MF_EINVAL;
  cudaError_t e = t.used ? cudaEventSynchronize(t.ev[t.used - 1]) : cudaSuccess;
  for (int i = 0; e == cudaSuccess && i + 1 < t.used; ++i) {
    if (t.kind[i] < 0) continue;
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, t.ev[i], t.ev[i + 1]);
    launches[t.kind[i]] += 1;
    total_ms[t.kind[i]] += ms;
  }
  const bool overflow = t.overflow;
  t.used = 0;
  t.overflow = false;
  if (e != cudaSuccess) {
    set_last_error("mf_profile_read", e);
    return MF_ECUDA;
  }
  if (overflow) {
    std::snprintf(g_last_error, sizeof(g_last_error), "mf_profile_read: more than %d launches since the last read",
                  LaunchTimer::kEvents - 1);
    return MF_ENOMEM;
  }
  return MF_OK;
}

int mf_set_conditions(mf_context* c, int t, const mf_conditions* cond) {
  if (!c || !cond || t < 0 || t >= MF_MAX_CTYPES) return MF_EINVAL;
  DevConditions d;
  int rc = make_dev_conditions(*cond, &d);
  if (rc) return rc;
  std::lock_guard<std::mutex> g(c->mu);
  c->cond[t] = d;
  c->cond_set[t] = 1;
  return upload_tables(c, t);
}

int mf_fit(mf_context* c, const mf_batch* b, const mf_options* o, void* stream) {
  FitArgs a;
  int rc = fill_args(c, b, o, &a);
  if (rc) return rc;
  if (b->n == 0) return MF_OK;
  return dispatch(c, a, o, (cudaStream_t)stream, false);
}

// Instrumented variant: same fit, plus the executed floating-point operation
// count of every channel in flops[n] (device pointer). Used to measure the
// algorithmic work of a workload; not part of the timed path.
int mf_fit_count_flops(mf_context* c, const mf_batch* b, const mf_options* o, double* flops, void* stream) {
  FitArgs a;
  int rc = fill_args(c, b, o, &a);
  if (rc) return rc;
  if (!flops) return MF_EINVAL;
  if (b->n == 0) return MF_OK;
  a.flops = flops;
  return dispatch(c, a, o, (cudaStream_t)stream, true);
}

// Chunk boundaries of a host-pointer fit: offs[0] = 0 < ... < offs[k] = n,
// returns k. Full chunks of B = MIXED_CHUNK channels with a ramp of B/4 and
// B/2 at both ends (with `taper`, B/2, B/4 and B/8 at the end): only the first
// chunk's copy-in and the last chunk's copy-out are not hidden under a fit
// (88 B in and 99 B out per channel; the link carries 211 GB/s host to
// device, 193 GB/s back, 327 GB/s both ways at once). Measured on 10M warm
// channels (e2e ms per step, device fit 7.55 ms at the time): 8.74 with this
// rule, 8.80 with B halved, 9.53 with B quartered, 9.02 without the ramp; the
// B/8 taper takes 0.03 ms more off the warm pipeline, where the last copy-out
// is on the critical path. Batches too small for the ramp are cut into up to
// eight equal chunks of at least B/8.
int host_chunks(int64_t n, int64_t* offs, bool taper) {
  constexpr int64_t B = int64_t(1) << 21, R = B / 8;  // the ramp's unit (2M channels)
  constexpr int64_t up[2] = {B / 4, B / 2};
  constexpr int64_t down[2][3] = {{B / 2, B / 4, 0}, {B / 2, B / 4, B / 8}};
  const int64_t* dn = down[taper ? 1 : 0];
  const int ndown = taper ? 3 : 2;
  const int64_t ramp_sum = up[0] + up[1] + dn[0] + dn[1] + dn[2];
  int k = 0;
  offs[0] = 0;
  if (n >= ramp_sum + B) {
    for (int64_t r : up) offs[k + 1] = offs[k] + r, ++k;
    const int64_t middle = n - ramp_sum;
    int64_t parts = (middle + B - 1) / B;  // beyond the event slots the middle chunks grow past B
    if (parts > mf_context::kHostChunks - 5) parts = mf_context::kHostChunks - 5;
    for (int64_t p = 0; p < parts; ++p) offs[k + 1] = offs[2] + middle * (p + 1) / parts, ++k;
    for (int j = 0; j < ndown; ++j) offs[k + 1] = offs[k] + dn[j], ++k;
  } else {
    int64_t parts = (n + R - 1) / R;
    if (parts > 8) parts = 8;
    if (parts < 1) parts = 1;
    for (int64_t p = 0; p < parts; ++p) offs[k + 1] = n * (p + 1) / parts, ++k;
  }
  return k;
}

// Host-pointer fit, pipelined: the batch is cut into chunks (host_chunks); the
// copy-in of chunk i+1 (h2d stream) and the copy-out of chunk i-1 (d2h stream)
// run under the fit of chunk i, ordered by events. With pinned host buffers
// the step costs about max(copies, fit) instead of their sum. Two shapes:
// - cold starts of the mixed and FP32 forms (fit 9-12 ms per 10M channels
//   against 5.7 ms of copies): even chunks fit on the context stream and odd
//   chunks on a second stream with its own workspace (lane 1), so
//   neighbouring fits overlap (one chunk's queue kernels, whose time is set by
//   their slowest channels, run beside the next chunk's search); chunk i + 2
//   reuses chunk i's lane on the same stream;
// - the warm start (fit 5.8 ms, as long as the copies): chunks fit in order
//   on one stream, so each chunk's copy-out starts as early as it can; the
//   copy-in of chunk i waits for the fit of chunk i - 2, leaving the link to
//   the copy-outs once the next two inputs are in; the last chunks taper to
//   B/8. Measured on 10M channels (e2e ms per step): warm 7.53 two lanes,
//   7.31 one lane with the throttle and the taper; cold FP32 9.74 two lanes vs
//   9.89 one, cold mixed 12.52 vs 13.29, ECAL/HCAL persistent FP32 10.21 vs
//   11.04.
// The FP64 form and per-kernel profiling keep one stream.
int mf_fit_host(mf_context* c, const mf_batch* hb, const mf_options* o) {
  if (!c || !hb) return MF_EINVAL;
  std::lock_guard<std::mutex> g(c->mu);
  const int64_t n = hb->n;
  if (n < 0) return MF_EINVAL;
  if (n == 0) return MF_OK;
  int rc = grow_staging(c, n, hb->sample_stride, hb->amp_stride);
  if (rc) return rc;
  {  // validate once on the whole batch before any copy
    mf_batch db = *hb;
    db.samples = c->d_samples;
    db.pederr = c->d_pederr;
    db.ctype = hb->ctype ? c->d_ctype : nullptr;
    db.amplitudes = c->d_amp;
    db.chi2 = c->d_chi2;
    FitArgs a;
    rc = fill_args(c, &db, o, &a);
    if (rc) return rc;
  }
  cudaError_t e = cudaSuccess;
  if (!c->h2d_stream) e = cudaStreamCreateWithFlags(&c->h2d_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess && !c->d2h_stream) e = cudaStreamCreateWithFlags(&c->d2h_stream, cudaStreamNonBlocking);
  for (int i = 0; i < mf_context::kHostChunks && e == cudaSuccess; ++i) {
    if (!c->in_done[i]) e = cudaEventCreateWithFlags(&c->in_done[i], cudaEventDisableTiming);
    if (e == cudaSuccess && !c->fit_done[i]) e = cudaEventCreateWithFlags(&c->fit_done[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    set_last_error("mf_fit_host: stream/event setup", e);
    return MF_ECUDA;
  }
  const bool warm = o->warm_start == MF_WARM_MLP;
  int64_t offs[mf_context::kHostChunks + 1];
  const int nchunks = host_chunks(n, offs, warm);
  const bool two = nchunks > 1 && !c->timer.ev && !warm &&
                   (o->precision == MF_PREC_MIXED || o->precision == MF_PREC_FP32);
  if (two) {
    rc = grow_lane1(c);
    if (rc) return rc;
    // the second stream starts after everything already queued on the context stream
    e = cudaEventRecord(c->fork, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream2, c->fork, 0);
  }
  const int ss = hb->sample_stride, as = hb->amp_stride;
  auto cp = [&](void* dst, const void* src, size_t bytes, cudaMemcpyKind k, cudaStream_t st) {
    if (e == cudaSuccess && src && dst && bytes) e = cudaMemcpyAsync(dst, src, bytes, k, st);
  };
  for (int i = 0; i < nchunks && e == cudaSuccess && rc == MF_OK; ++i) {
    const int64_t off = offs[i], m = offs[i + 1] - offs[i];
    // copy in (the warm start: at most two chunks ahead of the fits)
    if (warm && i >= 2 && e == cudaSuccess) e = cudaStreamWaitEvent(c->h2d_stream, c->fit_done[i - 2], 0);
    cp(c->d_samples + off * ss, hb->samples + off * ss, sizeof(double) * m * ss, cudaMemcpyHostToDevice, c->h2d_stream);
    cp(c->d_pederr + off, hb->pederr + off, sizeof(double) * m, cudaMemcpyHostToDevice, c->h2d_stream);
    if (hb->ctype) cp(c->d_ctype + off, hb->ctype + off, m, cudaMemcpyHostToDevice, c->h2d_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->in_done[i], c->h2d_stream);
    // fit
    const int lane = two ? (i & 1) : 0;
    cudaStream_t fs = lane ? c->stream2 : c->stream;
    if (e == cudaSuccess) e = cudaStreamWaitEvent(fs, c->in_done[i], 0);
    if (e != cudaSuccess) break;
    mf_batch db = *hb;
    db.n = m;
    db.samples = c->d_samples + off * ss;
    db.pederr = c->d_pederr + off;
    db.ctype = hb->ctype ? c->d_ctype + off : nullptr;
    db.amplitudes = c->d_amp + off * as;
    db.chi2 = c->d_chi2 + off;
    db.intime = hb->intime ? c->d_intime + off : nullptr;
    db.errors = hb->errors ? c->d_errors + off : nullptr;
    db.active_mask = hb->active_mask ? c->d_mask + off : nullptr;
    db.status = hb->status ? c->d_status + off : nullptr;
    db.iters = hb->iters ? c->d_iters + off : nullptr;
    FitArgs a;
    rc = fill_args(c, &db, o, &a);
    if (rc == MF_OK) rc = dispatch(c, a, o, fs, false, false, lane);
    if (rc != MF_OK) break;
    e = cudaEventRecord(c->fit_done[i], fs);
    // copy out
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->d2h_stream, c->fit_done[i], 0);
    cp(hb->amplitudes + off * as, c->d_amp + off * as, sizeof(double) * m * as, cudaMemcpyDeviceToHost, c->d2h_stream);
    cp(hb->chi2 + off, c->d_chi2 + off, sizeof(double) * m, cudaMemcpyDeviceToHost, c->d2h_stream);
    if (hb->intime) cp(hb->intime + off, c->d_intime + off, sizeof(double) * m, cudaMemcpyDeviceToHost, c->d2h_stream);
    if (hb->errors) cp(hb->errors + off, c->d_errors + off, sizeof(double) * m, cudaMemcpyDeviceToHost, c->d2h_stream);
    if (hb->active_mask)
      cp(hb->active_mask + off, c->d_mask + off, sizeof(uint16_t) * m, cudaMemcpyDeviceToHost, c->d2h_stream);
    if (hb->status) cp(hb->status + off, c->d_status + off, m, cudaMemcpyDeviceToHost, c->d2h_stream);
    if (hb->iters) cp(hb->iters + off, c->d_iters + off, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, c->d2h_stream);
  }
  // drain all three streams, whatever happened above
  const cudaError_t e1 = cudaStreamSynchronize(c->h2d_stream);
  cudaError_t e2 = cudaStreamSynchronize(c->stream);
  if (c->stream2) {
    const cudaError_t e4 = cudaStreamSynchronize(c->stream2);
    if (e2 == cudaSuccess) e2 = e4;
  }
  const cudaError_t e3 = cudaStreamSynchronize(c->d2h_stream);
  if (rc != MF_OK) return rc;
  if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
  if (e != cudaSuccess) {
    set_last_error("mf_fit_host", e);
    return MF_ECUDA;
  }
  if (c->mlp.infer_err) {
    // a bounded tensor-core wait of the warm-start inference gave up: those
    // channels were fitted from a cold start (same results), reported once
    unsigned flags = 0;
    e = cudaMemcpy(&flags, c->mlp.infer_err, sizeof(flags), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && flags) e = cudaMemset(c->mlp.infer_err, 0, sizeof(flags));
    if (e != cudaSuccess) {
      set_last_error("mf_fit_host", e);
      return MF_ECUDA;
    }
    if (flags & MLP_ERR_TIMEOUT) return MF_ETIMEOUT;
  }
  return MF_OK;
}

int mf_mlp_param_count(void) { return P_COUNT; }

int mf_mlp_init(mf_context* c, int ctype, uint64_t seed) {
  if (!c || ctype < 0 || ctype >= MF_MAX_CTYPES) return MF_EINVAL;
  std::lock_guard<std::mutex> g(c->mu);
  return mlp_init(c->mlp, c->device, ctype, seed);
}

int mf_mlp_train(mf_context* c, const mf_batch* d, const mf_mlp_train_params* p, float* epoch_loss, void* stream) {
  if (!c || !d || !p || !d->samples || !d->pederr || !d->amplitudes || p->epochs < 0) return MF_EINVAL;
  if (!c->mlp.ready) return MF_ENOTRAINED;
  const int t = c->mlp.set;
  if (!c->tab_ok[t] || c->tab[t].N != 10) return MF_EUNSUPPORTED;
  std::lock_guard<std::mutex> g(c->mu);
  return mlp_train(c->mlp, c->tab[t], d->n, d->sample_stride, d->samples, d->pederr, d->ctype, d->amplitudes,
                   d->amp_stride, *p, epoch_loss, (cudaStream_t)stream);
}

int mf_mlp_gradient(mf_context* c, const mf_batch* d, const mf_mlp_train_params* p, float* grads,
                    uint16_t* features_bf16, float* targets, float* loss) {
  if (!c || !d || !p || !grads || !features_bf16 || !targets || !loss || !d->amplitudes) return MF_EINVAL;
  if (!c->mlp.ready) return MF_ENOTRAINED;
  const int t = c->mlp.set;
  if (!c->tab_ok[t] || c->tab[t].N != 10) return MF_EUNSUPPORTED;
  std::lock_guard<std::mutex> g(c->mu);
  MlpGradProbe probe{grads, reinterpret_cast<__nv_bfloat16*>(features_bf16), targets, loss};
  return mlp_train(c->mlp, c->tab[t], d->n, d->sample_stride, d->samples, d->pederr, d->ctype, d->amplitudes,
                   d->amp_stride, *p, nullptr, c->stream, &probe);
}

int mf_mlp_get_weights(mf_context* c, float* host) {
  if (!c || !host) return MF_EINVAL;
  return mlp_get_weights(c->mlp, host);
}

int mf_mlp_set_weights(mf_context* c, const float* host) {
  if (!c || !host) return MF_EINVAL;
  std::lock_guard<std::mutex> g(c->mu);
  return mlp_set_weights(c->mlp, host);
}

int mf_mlp_test_stall(mf_context* c, int enable) {
  if (!c) return MF_EINVAL;
  std::lock_guard<std::mutex> g(c->mu);
  c->mlp.test_stall = enable ? 1 : 0;
  return MF_OK;
}

int mf_mlp_predict(mf_context* c, const mf_batch* b, uint16_t* mask, float* amp, float* logits, void* stream) {
  if (!c || !b || !mask || !amp || b->n < 0 || (b->n > 0 && (!b->samples || !b->pederr))) return MF_EINVAL;
  if (!c->mlp.ready) return MF_ENOTRAINED;
  const int t = c->mlp.set;
  if (!c->tab_ok[t] || c->tab[t].N != 10) return MF_EUNSUPPORTED;
  MlpInferArgs ia;
  fill_infer_args(c->mlp, c->tab[t], 0, &ia);
  ia.n = b->n;
  ia.sample_stride = b->sample_stride;
  ia.samples = b->samples;
  ia.pederr = b->pederr;
  ia.ctype = b->ctype;
  ia.warm_mask = mask;
  ia.warm_amp = amp;
  ia.warm_stride = 10;
  ia.logits = logits;
  cudaError_t e = launch_mlp_infer(ia, c->sms, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_last_error("mlp_infer launch", e);
    return MF_ECUDA;
  }
  return MF_OK;
}

int mf_table_operator(const mf_conditions* cond, uint32_t mask, double* whiten, double* pinv) {
  if (!cond) return MF_EINVAL;
  DevConditions d;
  int rc = make_dev_conditions(*cond, &d);
  if (rc) return rc;
  if (d.has_fpc || d.K > d.N) return MF_EUNSUPPORTED;
  if (mask == 0 || mask >= (1u << d.K)) return MF_EINVAL;
  HostTables h;
  rc = build_mixed_tables(d, &h);
  if (rc) return rc;
  if (whiten) {
    int w = 0;
    for (int i = 0; i < d.N; ++i)
      for (int j = 0; j < d.N; ++j) whiten[i * d.N + j] = j <= i ? h.W64[w++] : 0.;
  }
  if (pinv) {  // the rows of the set's columns, in ascending order
    const int p = __builtin_popcount(mask);
    std::memcpy(pinv, h.pinv64.data() + h.offset[mask], sizeof(double) * p * d.N);
  }
  return MF_OK;
}

int mf_build_pulse_matrix(const double* fullpulse, const int8_t* bxs, int N, int K, double* P) {
  if (!fullpulse || !bxs || !P || N < 1 || N > MF_MAX_SAMPLES || K < 1 || K > MF_MAX_PULSES) return MF_EINVAL;
  const int NF = N + 9;
  for (int k = 0; k < K; ++k) {
    const int bx = bxs[k];
    const int first = bx + 3 > 0 ? bx + 3 : 0;
    const int offset = 7 - 3 - bx;
    for (int i = 0; i < N; ++i) {
      double v = 0.;
      if (i >= first) {
        const int idx = i + offset;
        if (idx < 0 || idx >= NF) return MF_EINVAL;
        v = fullpulse[idx];
      }
      P[k * N + i] = v;
    }
  }
  return MF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// mf_fit_noalloc: the mixed-precision fit with its search -> judge hand-off in
// a fixed static device array instead of the context's cudaMalloc'd workspace.
//
// Who needs it: a module of a multi-threaded event-processing framework that
// owns the device memory through its own caching allocator. There cudaMalloc
// and cudaFree are not allowed on the per-event path: they synchronise the
// whole device (stalling the streams of every other event in flight) and take
// memory behind the pool's back. Such a caller allocates its channel buffers
// from its pool, sets the context up once at job start, and then calls this
// entry point, which allocates nothing.
//
// Limits: at most MF_NOALLOC_MAX_CHANNELS channels per call (larger batches
// are rejected with MF_EINVAL, never split or truncated); cold start only (no
// MLP warm start), no MINOS errors. The scratch is one array per device, so
// calls whose work overlaps on one device (two streams, two host threads, two
// contexts) race on it: serialise them, e.g. one stream per device.
// What must start at zero: only the two queue counters (judge -> fix,
// judge -> repair), and the search launch of every call writes them before
// the judge launches read them; the other scratch words are written before
// they are read within a call.
// ---------------------------------------------------------------------------

namespace {

constexpr int64_t kNoallocMax = MF_NOALLOC_MAX_CHANNELS;
constexpr size_t kAlignUp(size_t b) { return (b + 255) & ~size_t(255); }
// byte offsets of the hand-off arrays inside the scratch (each 256-byte aligned)
constexpr size_t kOffX = 0;                                                     // float [max][KMAX]
constexpr size_t kOffQueue = kOffX + kAlignUp(sizeof(float) * kNoallocMax * KMAX);  // int [max]
constexpr size_t kOffFixq = kOffQueue + kAlignUp(sizeof(int) * kNoallocMax);       // int [max]
constexpr size_t kOffMask = kOffFixq + kAlignUp(sizeof(int) * kNoallocMax);        // uint16 [max]
constexpr size_t kOffCount = kOffMask + kAlignUp(sizeof(uint16_t) * kNoallocMax);  // uint16 [max]
constexpr size_t kOffAdd = kOffCount + kAlignUp(sizeof(uint16_t) * kNoallocMax);    // uint16 [max]
constexpr size_t kOffQcount = kOffAdd + kAlignUp(sizeof(uint16_t) * kNoallocMax);   // unsigned [2]
constexpr size_t kNoallocBytes = kOffQcount + 256;  // 7,078,144 bytes for 131,072 channels

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kMaxDevices] = {};

// Address of this device's scratch, resolved once per device (the device must
// be current). The first call on a device resolves it; make that call before
// any stream capture on the device begins. The address is cached for the
// process: a cudaDeviceReset between calls would leave it stale.
int noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return MF_EINVAL;
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      set_last_error("mf_fit_noalloc: cudaGetSymbolAddress of the static scratch", e);
      return MF_ECUDA;
    }
    g_noalloc_ptr[device] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_ptr[device];
  return MF_OK;
}

}  // namespace

extern "C" int mf_fit_noalloc(mf_context* c, const mf_batch* b, const mf_options* o, void* stream) {
  FitArgs a;
  int rc = fill_args(c, b, o, &a);
  if (rc) return rc;
  if ((o->precision != MF_PREC_MIXED && o->precision != MF_PREC_FP32) || o->warm_start != MF_WARM_NONE ||
      o->compute_errors || o->schedule != MF_SCHED_GRID) {
    std::snprintf(g_last_error, sizeof(g_last_error),
                  "mf_fit_noalloc: only the mixed or FP32 precision, cold start, grid schedule, no errors");
    return MF_EUNSUPPORTED;
  }
  if (b->n > kNoallocMax) {
    std::snprintf(g_last_error, sizeof(g_last_error),
                  "mf_fit_noalloc: batch of %lld channels exceeds MF_NOALLOC_MAX_CHANNELS = %lld; split it",
                  (long long)b->n, (long long)kNoallocMax);
    return MF_EINVAL;
  }
  for (int t = 0; t < a.n_ctypes; ++t)
    if (!c->tab_ok[t] || c->cond[t].has_fpc) {
      std::snprintf(g_last_error, sizeof(g_last_error),
                    "mf_fit_noalloc: condition set %d has no passive-set tables (shape or pulse covariance)", t);
      return MF_EUNSUPPORTED;
    }
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) {
    set_last_error("mf_fit_noalloc: cudaGetDevice", e);
    return MF_ECUDA;
  }
  if (cur != c->device) {
    std::snprintf(g_last_error, sizeof(g_last_error),
                  "mf_fit_noalloc: the context's device %d is not the current device %d", c->device, cur);
    return MF_EINVAL;
  }
  unsigned char* scratch = nullptr;
  rc = noalloc_scratch(cur, &scratch);
  if (rc) return rc;
  if (b->n == 0) return MF_OK;
  MixedArgs m;
  std::memset(&m, 0, sizeof(m));
  for (int t = 0; t < a.n_ctypes; ++t) fill_dev_mixed(c, t, &m.tab[t]);
  m.n_ctypes = a.n_ctypes;
  m.skip_set = -1;
  m.warm_set = -1;
  m.n = a.n;
  m.sample_stride = a.sample_stride;
  m.amp_stride = a.amp_stride;
  m.max_iter32 = 12;  // the search and repair limits of mf_fit's mixed precision
  m.max_iter64 = o->max_iter_nnls > 0 ? o->max_iter_nnls : 1;
  m.tol32 = 1e-5f;
  m.eps = o->nnls_eps;
  m.eps32 = float(o->nnls_eps);
  m.samples = a.samples;
  m.pederr = a.pederr;
  m.ctype = a.ctype;
  m.amplitudes = a.amplitudes;
  m.chi2 = a.chi2;
  m.intime = a.intime;
  m.active_mask = a.active_mask;
  m.status = a.status;
  m.iters = a.iters;
  m.ws_x = reinterpret_cast<float*>(scratch + kOffX);
  m.ws_queue = reinterpret_cast<int*>(scratch + kOffQueue);
  m.ws_fixq = reinterpret_cast<int*>(scratch + kOffFixq);
  m.ws_mask = reinterpret_cast<uint16_t*>(scratch + kOffMask);
  m.ws_count = reinterpret_cast<uint16_t*>(scratch + kOffCount);
  m.ws_add = reinterpret_cast<uint16_t*>(scratch + kOffAdd);
  m.ws_qcount = reinterpret_cast<unsigned*>(scratch + kOffQcount);
  m.sms = c->sms;
  m.judge_df = o->precision == MF_PREC_FP32 ? 1 : 0;
  e = launch_fit_mixed(m, o->block_size, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_last_error("mf_fit_noalloc launch", e);
    return MF_ECUDA;
  }
  return MF_OK;
}
