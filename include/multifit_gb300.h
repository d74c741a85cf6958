/*
 * multifit_gb300.h -- C ABI of the GB300 multifit engine.
 *
 * The engine fits, per detector channel, N ADC samples (N <= 10) with a
 * non-negative sum of K (<= 10) time-shifted pulse templates under the
 * noise covariance C = pederr^2 * samplecor (+ the amplitude-dependent
 * pulse-shape term when a fullpulsecov is given). It returns per-BX
 * amplitudes, chi2, the final passive (active-amplitude) set, a status word
 * and iteration counters, as the reference's per-channel fit does:
 *
 *   bool PulseChiSqSNNLS::DoFit(samples, samplecor, pederr, bxs, fullpulse,
 *                               fullpulsecov)      multifit_cpu/interface/PulseChiSqSNNLS.h:13-18
 *   X(), ChiSq(), BXs(), Errors()                  multifit_cpu/interface/PulseChiSqSNNLS.h:23-27
 *
 * and the reference GPU batch entry
 *
 *   std::vector<Output> doFitWrapper(std::vector<DoFitArgs> const&)
 *                                                  multifit_gpu/interface/PulseChiSqSNNLSWrapper.h:11
 *
 * Differences at the boundary, by design:
 *  - inputs are structure-of-arrays per channel; the per-channel conditions
 *    (pulse matrix, sample correlation, BX list, pulse covariance) that every
 *    reference DoFitArgs repeats (multifit_gpu/interface/DeviceData.h:6-26)
 *    are passed once per batch as up to MF_MAX_CTYPES condition sets, and
 *    each channel names its set;
 *  - the caller owns every buffer; device entry points allocate nothing and
 *    never synchronise (mf_fit_host is the synchronous host-pointer variant);
 *  - errors are returned as codes, never printed
 *    (the reference prints them: multifit_gpu/src/PulseChiSqSNNLSWrapper.cu:33-39).
 *
 * Matrices are column-major like the reference's Eigen types: element (i,j)
 * of an R x C matrix sits at [j*R + i].
 */
#ifndef MULTIFIT_GB300_H
#define MULTIFIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MF_ABI_VERSION 1
#define MF_MAX_SAMPLES 10
#define MF_MAX_PULSES 10
#define MF_MAX_CTYPES 2
#define MF_FULLPULSE_MAX (MF_MAX_SAMPLES + 9)

/* Return codes of every entry point. */
enum mf_rc {
  MF_OK = 0,
  MF_EINVAL = 1,       /* bad argument (null pointer, size out of range, bad option) */
  MF_ECUDA = 2,        /* a CUDA runtime call failed; mf_last_error() has the text */
  MF_ETIMEOUT = 3,     /* a bounded device-side wait gave up */
  MF_ENOMEM = 4,       /* context workspace could not be allocated */
  MF_EUNSUPPORTED = 5, /* option combination not built */
  MF_ENOTRAINED = 6    /* MLP warm start requested before weights were set */
};

/* Per-channel status bits (mf_batch.status). 0 = converged fit. */
enum mf_channel_status {
  MF_CH_NNLS_MAXITER = 1,  /* last FNNLS call stopped at max_iter_nnls before KKT */
  MF_CH_OUTER_MAXITER = 2, /* outer chi2 loop stopped at max_iter_outer */
  MF_CH_NONFINITE = 4,     /* non-finite amplitude or chi2 (e.g. non-PD covariance) */
  MF_CH_BADINPUT = 8       /* non-finite sample or pederr, or bad condition index */
};

/* Arithmetic of the fit. MF_PREC_MIXED and MF_PREC_FP32 return each channel's
 * NNLS optimum (KKT point) within 1e-4 of the FP64 fit run to convergence.
 * With no pulse covariance and errors off they fit through the passive-set
 * tables of the condition set (N = K = 10 or 8). Otherwise the batch takes
 * the per-channel form: the outer chi2 loop's first iteration (covariance
 * pederr^2 samplecor, the tables' problem) through the tables, then the FP64
 * fit from its amplitudes and chi2 -- the amplitude-dependent covariance, the
 * FNNLS from their support, the stopping rule, the MINOS-like refits -- on the
 * grid schedule. Shapes without tables are fitted in FP64 throughout. */
enum mf_precision {
  MF_PREC_FP64 = 0,  /* plain FP64, bit-identical to the CPU oracle's canonical order */
  MF_PREC_MIXED = 1, /* FP32 search and screen; FP64 refinement solve, residual and chi2 (the judge) */
  MF_PREC_FP32 = 2   /* FP32 throughout: the judge's solve, residual and chi2 in double-float FP32
                        arithmetic (~2^-48 per operation); FP64 only for the rare repaired channels */
};

/* How channels are scheduled onto the GPU. */
enum mf_schedule {
  MF_SCHED_GRID = 0,      /* one thread per channel, one launch */
  MF_SCHED_PERSISTENT = 1 /* persistent blocks that take channels from a work counter */
};

/* Start of the FNNLS active-set loop. */
enum mf_warm {
  MF_WARM_NONE = 0, /* reference start: empty passive set, x = previous amplitudes */
  MF_WARM_MLP = 1   /* passive set and amplitudes predicted by the trained MLP */
};

/* One set of fit conditions, shared by every channel that names it. */
typedef struct mf_conditions {
  int32_t nsamples;                          /* N, 1..10 */
  int32_t npulses;                           /* K, 1..10 */
  double pulse_matrix[MF_MAX_SAMPLES * MF_MAX_PULSES]; /* N x K column-major: (i,k) at [k*N+i] */
  double noise_cor[MF_MAX_SAMPLES * MF_MAX_SAMPLES];   /* N x N samplecor, (i,j) at [j*N+i]; lower triangle read */
  int8_t bxs[MF_MAX_PULSES];                 /* BX offset of each pulse column */
  int32_t has_fullpulsecov;                  /* 0: no pulse-shape covariance term */
  double fullpulsecov[MF_FULLPULSE_MAX * MF_FULLPULSE_MAX]; /* (N+9) x (N+9) column-major */
} mf_conditions;

/* How each FNNLS call starts from the previous amplitudes. */
enum mf_nnls_start {
  /* The reference's start: empty passive set, x = the previous amplitudes
   * (nnls/src/inplace_fnnls.cu:97, multifit_cpu/src/PulseChiSqSNNLS.cpp:258).
   * Entries outside the passive set keep stale values, and with the absolute
   * nnls_eps below the round-off of w a later outer iteration can stop in a
   * state that is not the NNLS optimum. Bit-identical to the oracle. */
  MF_START_REFERENCE = 0,
  /* Passive set seeded with the support of the previous amplitudes, made
   * feasible by the inner loop, then the reference loop: a proper FNNLS warm
   * start. The first outer iteration (x = 0) is the same as the reference's. */
  MF_START_SUPPORT = 1
};

/* Fit options. mf_default_options() gives the multifit_cpu settings. */
typedef struct mf_options {
  int32_t max_iter_nnls;  /* FNNLS iteration cap: 10 as multifit_cpu (PulseChiSqSNNLS.cpp:243), 1000 as multifit_gpu */
  int32_t max_iter_outer; /* outer chi2 iterations: 50 (PulseChiSqSNNLS.cpp:153) */
  double dchi2_tol;       /* stop when |chi2 - chi2_prev| < tol: 1e-3 (PulseChiSqSNNLS.cpp:162) */
  double nnls_eps;        /* FNNLS stop when max w < eps: 1e-11 (PulseChiSqSNNLS.cpp:242) */
  int32_t nnls_start;     /* enum mf_nnls_start */
  int32_t precision;      /* enum mf_precision */
  int32_t schedule;       /* enum mf_schedule */
  int32_t warm_start;     /* enum mf_warm */
  int32_t compute_errors; /* 1: MINOS-like in-time uncertainty (DoFit, PulseChiSqSNNLS.cpp:75-146) */
  int32_t block_size;     /* threads per block, a multiple of 32; grid schedule at most 128, persistent
                             at most 512 (MF_EINVAL beyond); 0 = tuned default */
  int32_t blocks_per_sm;  /* persistent schedule: cap on resident blocks per SM; 0 = the occupancy limit */
  int32_t channels_per_warp; /* persistent schedule, FP32 search: 1, 2, 4, 8 or 32 channels per warp
                                (32 / that many lanes per channel); 0 = tuned (mf_autotune) or 32 */
} mf_options;

/* A batch of channels. Every pointer is a DEVICE pointer for mf_fit and a
 * HOST pointer for mf_fit_host. Optional outputs may be NULL. */
typedef struct mf_batch {
  int64_t n;                 /* number of channels */
  int32_t sample_stride;     /* doubles between consecutive channels of samples (>= N of every set) */
  int32_t amp_stride;        /* doubles between consecutive channels of amplitudes (>= K of every set) */
  const double* samples;     /* [n][sample_stride] pedestal-subtracted ADC samples */
  const double* pederr;      /* [n] noise scale: C = pederr^2 * samplecor */
  const uint8_t* ctype;      /* [n] condition-set index, or NULL (all channels use set 0) */
  double* amplitudes;        /* [n][amp_stride] fitted amplitude per pulse column (unpermuted, X()) */
  double* chi2;              /* [n] ChiSq() */
  double* intime;            /* [n] amplitude of the in-time column (first k with bxs[k]==0), or NULL */
  double* errors;            /* [n] in-time uncertainty (Errors()), or NULL; needs compute_errors */
  uint16_t* active_mask;     /* [n] bit k set: amplitude k > 0 (the support of X()), or NULL */
  uint8_t* status;           /* [n] enum mf_channel_status bits, or NULL */
  int32_t* iters;            /* [n] outer | fnnls<<8 | inner<<20 counts (saturating), or NULL */
} mf_batch;

typedef struct mf_context mf_context;

/* Library and context --------------------------------------------------- */
int mf_abi_version(void);
const char* mf_rc_string(int rc);
/* Text of the last CUDA error seen by this thread (empty if none). */
const char* mf_last_error(void);
void mf_default_options(mf_options* opt);

/* Creates a context bound to a CUDA device and allocates its workspace. */
int mf_create(mf_context** out, int device);
void mf_destroy(mf_context* ctx);
/* Copies a condition set into the context. For a set without a pulse
 * covariance it also builds, once, the tables of the mixed-precision and
 * warm-start forms (whitening operator and the least-squares operator of every
 * passive set, ~0.6 MB for N = K = 10) and uploads them to the device;
 * with the first such set it allocates the context's workspace for those
 * forms (one chunk of 16,777,216 channels: ~1 GB, plus 672 MB for the warm
 * start's predictions when the network is initialised)
 * (synchronous; not a hot-path call). */
int mf_set_conditions(mf_context* ctx, int ctype, const mf_conditions* cond);

/* Fits a batch whose buffers are in device memory; asynchronous on `stream`
 * (a cudaStream_t; NULL = legacy default stream). No allocation, no sync. */
int mf_fit(mf_context* ctx, const mf_batch* batch, const mf_options* opt, void* stream);

/* Same fit as mf_fit, additionally writing the executed floating-point
 * operation count of every channel to flops[n] (device pointer; an FMA counts
 * 2, add/sub/mul/div/sqrt 1): every FP64 and no other operation for the plain
 * FP64 precision (an instrumented, slower build, never the timed path), the
 * FP64 operations (the bound of that kernel) for the mixed precision. */
int mf_fit_count_flops(mf_context* ctx, const mf_batch* batch, const mf_options* opt, double* flops, void* stream);

/* Same fit as mf_fit with the mixed or FP32 precision (cold start, grid
 * schedule, no errors), for callers that may not allocate device memory per call: a module
 * of a multi-threaded event-processing framework whose caching allocator owns
 * the device memory, where cudaMalloc/cudaFree would synchronise the device
 * under every other event in flight. The search-to-judge hand-off lives in a
 * static device array (about 6.8 MB per device) instead of the context's
 * workspace; the call allocates nothing. No counterpart in the reference
 * (multifit_cpu allocates nothing on the device).
 *  - n > MF_NOALLOC_MAX_CHANNELS: MF_EINVAL, mf_last_error says why.
 *  - The context's device must be current. The first call on a device
 *    resolves the scratch address (cudaGetSymbolAddress): make it before any
 *    stream capture on that device begins. The address is kept for the life
 *    of the process: do not cudaDeviceReset a device between calls.
 *  - One scratch per device: calls that overlap on a device (other streams,
 *    threads or contexts) race on it; serialise them.
 *  - The only scratch words that must start at zero (the two queue counters)
 *    are written by the call itself before they are read. */
#define MF_NOALLOC_MAX_CHANNELS 131072
int mf_fit_noalloc(mf_context* ctx, const mf_batch* batch, const mf_options* opt, void* stream);

/* Autotuner of the persistent schedule (the uneven ECAL/HCAL batches). One
 * point of the sweep: */
typedef struct mf_tune_point {
  int32_t block_size;        /* threads per block of the FP32 search: 64, 128, 256, 512 */
  int32_t channels_per_warp; /* channels a warp of the FP32 search fits at once: 1, 2, 4, 8, 32 */
  double ms;                 /* best of 3 timed fits of the batch (CUDA events), after one warm-up */
} mf_tune_point;
#define MF_TUNE_POINTS 20
/* Sweeps block_size x channels_per_warp for opt (precision MF_PREC_MIXED or
 * MF_PREC_FP32, any warm start) on the given device batch (its outputs are overwritten), keeps
 * the fastest in the context (used when a persistent-schedule fit leaves
 * block_size / channels_per_warp at 0) and writes up to max_points points.
 * Synchronous. The reference has no tuner (its launch shape is fixed:
 * multifit_gpu/src/PulseChiSqSNNLSWrapper.cu:29-31, 256 threads per block). */
int mf_autotune(mf_context* ctx, const mf_batch* batch, const mf_options* opt, mf_tune_point* points,
                int max_points, int* n_points);

/* Per-kernel timing of fits (instrumentation, off by default). The GB300
 * counterpart of the reference's -DPROFILE timing around the batch (VTune
 * __itt_resume/__itt_pause and std::chrono, multifit_cpu/src/multifit.cpp:
 * 231-246): while enabled, every fit records a CUDA event on its stream before
 * each kernel launch and after its last one (8,192 events per read). */
enum mf_kernel_kind {
  MF_K_FIT_FP64 = 0,  /* fit_fp64_kernel: the plain FP64 fit */
  MF_K_MLP_INFER = 1, /* mlp_infer_tc_kernel: warm-start predictions (tcgen05) */
  MF_K_SEARCH = 2,    /* search_kernel / search_persist: FP32 active-set search */
  MF_K_JUDGE = 3,     /* judge_kernel / judge_persist: FP64 solve, residual, KKT test, chi2 */
  MF_K_REPAIR = 4,    /* repair_kernel / repair_persist: FP64 FNNLS of the channels the judge queued */
  MF_K_PARTITION = 5, /* partition_kernel: per-set channel lists of the persistent schedule */
  MF_K_REJUDGE = 6,   /* judge_fixed_kernel / judge_fixed_persist: the judge of the channels the fix changed */
  MF_K_FIX = 7,       /* fix_kernel / fix_persist: FP32 FNNLS step of the channels queued for it */
  MF_K_SCREEN = 8,    /* screen_kernel / screen_persist: FP32 double-float KKT screen (cold starts) */
  MF_K_COUNT = 9
};
/* enable != 0 creates the context's event pool (and clears it); 0 frees it. */
int mf_profile(mf_context* ctx, int enable);
/* Waits for the recorded fits, writes the launch count and the summed device
 * time (ms) of every kernel kind into launches[MF_K_COUNT] and
 * total_ms[MF_K_COUNT], and clears the record. MF_ENOMEM if more launches
 * were made than the pool holds (the counts cover the recorded ones). */
int mf_profile_read(mf_context* ctx, int32_t* launches, double* total_ms);

/* Same fit with HOST buffers: copies inputs to the context's device staging
 * area, fits, copies results back and synchronises. Grows the staging area
 * when the batch is larger than any before it. */
int mf_fit_host(mf_context* ctx, const mf_batch* host_batch, const mf_options* opt);

/* Builds the N x K pulse matrix from a (N+9)-sample fullpulse and the BX
 * list with the reference's sliding-window rule
 * (multifit_cpu/src/PulseChiSqSNNLS.cpp:49-62): P(i,k) = fullpulse(i+4-bx_k)
 * for i >= max(0, bx_k+3), else 0. Host-only. */
int mf_build_pulse_matrix(const double* fullpulse, const int8_t* bxs, int nsamples, int npulses,
                          double* pulse_matrix);

/* Learned warm start ------------------------------------------------------
 * A small MLP (16 -> 128 -> 128 -> 32, ReLU, BF16 tensor-core GEMMs with FP32
 * accumulate, FP32 master weights) predicts from a channel's whitened
 * samples and noise scale its passive set and amplitudes; the mixed form
 * (warm_start = MF_WARM_MLP) then starts FNNLS there and still runs it to KKT
 * convergence with the FP64 judge, so a wrong prediction costs iterations,
 * never accuracy. It serves one condition set with N = K = 10; channels of
 * other sets start cold. No counterpart in the reference. */
typedef struct mf_mlp_train_params {
  int32_t epochs;
  int32_t batch;      /* multiple of 64 */
  float lr;           /* Adam learning rate */
  float amp_weight;   /* weight of the amplitude loss against the passive-set BCE */
} mf_mlp_train_params;

int mf_mlp_param_count(void);
/* Allocates the network (He-normal init from `seed`) for condition set `ctype`. */
int mf_mlp_init(mf_context* ctx, int ctype, uint64_t seed);
/* Trains on device data: batch.samples/pederr/ctype are the inputs and
 * batch.amplitudes holds their converged fits (the targets). Writes the mean
 * loss of each epoch to epoch_loss (host, may be NULL). Synchronous. Its
 * GEMMs run on the tensor cores (tcgen05) with bounded waits: MF_ETIMEOUT if
 * one gave up (the network is then left untrained). */
int mf_mlp_train(mf_context* ctx, const mf_batch* data, const mf_mlp_train_params* p, float* epoch_loss, void* stream);
/* Gradient check: one forward/backward on the first p->batch channels of
 * `data` without an update. Host outputs: grads[mf_mlp_param_count()], the
 * bf16 bit patterns of the input features [batch][16], the targets
 * [batch][20] (10 support bits, 10 scaled amplitudes) and the batch loss. */
int mf_mlp_gradient(mf_context* ctx, const mf_batch* data, const mf_mlp_train_params* p, float* grads,
                    uint16_t* features_bf16, float* targets, float* loss);
int mf_mlp_get_weights(mf_context* ctx, float* host_params);
int mf_mlp_set_weights(mf_context* ctx, const float* host_params);
/* Inference on device pointers: predicted passive set mask[n], amplitudes
 * amp[n][10] (GeV) and optionally the raw outputs logits[n][32]. */
int mf_mlp_predict(mf_context* ctx, const mf_batch* batch, uint16_t* mask, float* amp, float* logits, void* stream);
/* Test hook of the inference's timeout path (off by default). While enabled,
 * every inference wait first waits, for at most 1 ms, on an mbarrier nothing
 * arrives on: it gives up, the error is recorded (the next mf_fit_host
 * returns MF_ETIMEOUT), the tensor-core work in flight drains, and the
 * affected channels are fitted from a cold start (same results). */
int mf_mlp_test_stall(mf_context* ctx, int enable);

/* Host-only view of the mixed-form tables of a condition set (for checks):
 * whiten [N][N] row-major = L_R^-1 with L_R = chol(samplecor); pinv [p][N]
 * row-major = the least-squares operator of the passive set `mask` (columns in
 * ascending order, p = popcount(mask)). Either output may be NULL. */
int mf_table_operator(const mf_conditions* cond, uint32_t mask, double* whiten, double* pinv);

/* Synthetic channels ---------------------------------------------------- */

/* Condition-set kinds of the synthetic generator. */
enum mf_synth_kind {
  MF_SYNTH_ECAL = 0, /* N=K=10, CRRC4 (t/43ns)^4 e^{-t/43ns} peak 1, in-time sample 5, rho=0.7, sigma=0.044 */
  MF_SYNTH_HCAL = 1  /* N=K=8, (t/10ns)^2 e^{-t/10ns} peak 1, in-time sample 3, rho=0.3, sigma=0.8 */
};

typedef struct mf_synth_params {
  int64_t n;             /* channels */
  uint64_t seed;         /* Philox key: every channel is a pure function of (seed, channel index) */
  int32_t intime_log;    /* 0: in-time amplitude uniform in [lo,hi]; 1: log-uniform */
  double intime_lo, intime_hi;
  double pileup_mean;    /* Poisson mean of hits per out-of-time BX; < 0: per channel U[0, -pileup_mean] */
  double pileup_hit_mean;/* mean of the exponential hit energy */
  double hcal_fraction;  /* probability that a channel uses set 1 (HCAL); 0 = ECAL only */
} mf_synth_params;

/* Fills `cond` and the noise scale `sigma` of a synthetic condition set. */
int mf_synth_conditions(int kind, mf_conditions* cond, double* sigma);

/* Generates channels [first, first+count) of the stream defined by `p` into
 * samples [count][sample_stride], pederr [count], ctype [count] (may be NULL
 * when hcal_fraction == 0) and truth [count][truth_stride] (may be NULL).
 * on_device != 0: pointers are device pointers and the generator runs as a
 * kernel on `stream`; 0: host pointers, host threads. Host and device
 * streams agree to within the last bits of the libm functions used. */
int mf_synth_generate(const mf_synth_params* p, int64_t first, int64_t count, int sample_stride,
                      double* samples, double* pederr, uint8_t* ctype, double* truth, int truth_stride,
                      int on_device, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MULTIFIT_GB300_H */
