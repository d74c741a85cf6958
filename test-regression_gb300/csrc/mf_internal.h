// Internal declarations shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "multifit_gb300.h"

namespace mfgb {

constexpr int KMAX = 10;
constexpr int NFMAX = MF_FULLPULSE_MAX;

// Device copy of one condition set, passed to kernels by value (constant bank).
struct DevConditions {
  int N, K;
  int intime_col;                // first k with bxs[k] == 0, or -1
  int has_fpc;
  double P[KMAX * KMAX];         // N x K column-major
  double R[KMAX * KMAX];         // N x N column-major
  int8_t bxs[KMAX];
  int8_t fz[KMAX];               // first structurally non-zero row of column k (N if all zero)
  double fpc[NFMAX * NFMAX];     // (N+9) x (N+9) column-major, valid when has_fpc
};

struct DevOptions {
  int max_iter_nnls;
  int max_iter_outer;
  double dchi2_tol;
  double nnls_eps;
  int nnls_start;
  int compute_errors;
};

// Everything a fit kernel needs, passed by value.
struct FitArgs {
  DevConditions cond[MF_MAX_CTYPES];
  int n_ctypes;
  DevOptions opt;
  int64_t n;
  int sample_stride;
  int amp_stride;
  const double* samples;
  const double* pederr;
  const uint8_t* ctype;
  double* amplitudes;
  double* chi2;
  double* intime;
  double* errors;
  uint16_t* active_mask;
  uint8_t* status;
  int32_t* iters;
  double* flops;  // optional per-channel executed-flop count (instrumented build only)
  // 1: the outputs hold the amplitudes, chi2 and status of a first outer
  // iteration done elsewhere (the per-channel form's passive-set tables);
  // 2: ... of the FP64 kernel's own first iteration, with its FNNLS counters
  // in iters and its executed flops in flops (fit_core.cuh ChannelFit)
  int seeded;
  int sms;  // the device's SM count (the FP64 kernel launches one wave of resident blocks)
};

// Status bits (mirror of enum mf_channel_status).
enum : uint8_t { CH_NNLS_MAXITER = 1, CH_OUTER_MAXITER = 2, CH_NONFINITE = 4, CH_BADINPUT = 8 };

// Launchers (fit_fp64.cu).
// Per-kernel launch timing of fits (mf_profile): a CUDA event recorded on the
// launch stream before every kernel launch and after a fit's last launch; the
// time between two consecutive events belongs to the kernel launched after
// the first. Off unless enabled; the pool is created by mf_profile.
struct LaunchTimer {
  static constexpr int kEvents = 8192;
  cudaEvent_t* ev = nullptr;  // [kEvents]
  int8_t kind[kEvents];       // MF_K_* of the launch that follows event i; -1: end of a fit
  int used = 0;
  bool overflow = false;
  void mark(int k, cudaStream_t s) {
    if (!ev) return;
    if (used >= kEvents) {
      overflow = true;
      return;
    }
    if (cudaEventRecord(ev[used], s) != cudaSuccess) {
      overflow = true;
      return;
    }
    kind[used++] = int8_t(k);
  }
};

cudaError_t launch_fit_fp64(const FitArgs& a, int block, cudaStream_t s, bool instrumented,
                            LaunchTimer* tm = nullptr);

// Host tables of one condition set for the mixed / warm forms (tables.cu).
struct HostTables {
  int N = 0, K = 0;
  double W64[KMAX * (KMAX + 1) / 2];  // L_R^-1, packed lower rows
  float W32[KMAX * (KMAX + 1) / 2];
  float W32lo[KMAX * (KMAX + 1) / 2];  // W = W32 + W32lo to ~2^-48 (double-float)
  double G64[KMAX * KMAX];            // G = L_R^-1 P, N x K column-major
  float G32[KMAX * KMAX];
  float G32lo[KMAX * KMAX];
  float P32[KMAX * KMAX];             // P = P32 + P32lo to ~2^-48 (double-float), N x K column-major
  float P32lo[KMAX * KMAX];
  double H64[KMAX * KMAX];            // G^T G, row-major ld KMAX
  float H32[KMAX * KMAX];
  double gnorm2[KMAX];                // |G_k|^2
  int gfz[KMAX];                      // first structurally non-zero row of G_k
  std::vector<int> offset;            // per passive-set mask: offset of its p x N pseudo-inverse
  std::vector<double> pinv64;
  std::vector<float> pinv32;
  std::vector<float> pinv32lo;        // pinv64 = pinv32 + pinv32lo to ~2^-48
  std::vector<float> pinv2;           // element e as the pair (pinv32[e], pinv32lo[e]) at [2e], [2e + 1],
                                      // then G column by column as pairs (G32, G32lo) from [g2_off]
  int g2_off = 0;
};
int build_mixed_tables(const DevConditions& c, HostTables* t);

// Device view of one condition set's tables, passed by value.
struct DevMixed {
  int N, K, intime_col;
  double W64[KMAX * (KMAX + 1) / 2];
  float W32[KMAX * (KMAX + 1) / 2];
  float W32lo[KMAX * (KMAX + 1) / 2];
  double G64[KMAX * KMAX];
  double H64[KMAX * KMAX];
  float G32[KMAX * KMAX];
  float G32lo[KMAX * KMAX];
  float P32[KMAX * KMAX];
  float P32lo[KMAX * KMAX];
  float H32[KMAX * KMAX];
  float gnorm32[KMAX];
  int8_t gfz[KMAX];
  int zero_row;  // offset of an all-zero row after the last operator
  const int* offset;
  const double* pinv64;
  const float* pinv32;
  const float* pinv32lo;
  const float* pinv2;  // (hi, lo) pairs; a row of an even N starts on 16 bytes
  const float* g2;     // G as (hi, lo) pairs, column k at [2 k N] (inside the pinv2 buffer)
  const double* g64;   // G in FP64, column k at [k N], in global memory: the FP64 judge reads a
                       // different column in every lane, which the constant bank would serialise
};

struct MixedArgs {
  DevMixed tab[MF_MAX_CTYPES];
  int n_ctypes;
  int skip_set;  // condition set left to another launch (-1: none)
  int64_t n;
  int sample_stride, amp_stride;
  int max_iter32, max_iter64;
  float tol32;
  double eps;
  float eps32;  // eps rounded to float (the double-float judge's KKT tolerance)
  const double* samples;
  const double* pederr;
  const uint8_t* ctype;
  const uint16_t* warm_mask;  // learned warm start: predicted passive set, or null
  int warm_set;               // condition set the predictions belong to
  const float* warm_amp;      // predicted amplitudes [n][warm_stride]
  int warm_stride;
  double* amplitudes;
  double* chi2;
  double* intime;
  uint16_t* active_mask;
  uint8_t* status;
  int32_t* iters;
  double* flops;  // optional per-channel executed FP64 flops
  // hand-off from the FP32 search to the FP64 judge (context workspace)
  uint16_t* ws_mask;
  uint16_t* ws_count;
  float* ws_x;
  int* ws_queue;           // channels the judge queues for the FP64 repair
  int* ws_fixq;            // channels queued for the FP32 fix (their index in the chunk)
  uint16_t* ws_add;        // per channel: the columns the fix adds (written with its queue entry)
  unsigned* ws_qcount;     // [0] repair queue, [1] fix queue sizes (zeroed by the search launch)
  int sms;
  // persistent schedule (fit_sched.cu): per-set channel lists [MF_MAX_CTYPES][MIXED_CHUNK]
  // and SCHED_WORDS counters (list sizes, work counters, repair-queue sizes)
  int* ws_list;
  unsigned* ws_sched;
  int blocks_per_sm;       // cap on resident blocks per SM (0: the occupancy limit)
  int list_identity;       // one condition set, no ctype: the list is 0..n-1 (no partition pass)
  int judge_df;            // MF_PREC_FP32: the judge in double-float FP32 arithmetic instead of FP64
};
constexpr int SCHED_WORDS = 32;
// Channels per chunk of a mixed fit (the size of the hand-off workspace,
// 62 B per channel: 1 GB, and 672 MB of warm-start predictions). A chunk's
// queue kernels (fix, second judge, repair) hold a few per cent of its
// channels and are latency-bound: fewer, larger chunks give them more warps
// to hide their latency behind (10M warm channels: 5.24 ms per fit in chunks
// of 2M, 4.96 ms in chunks of 4M).
constexpr int64_t MIXED_CHUNK = int64_t(1) << 24;
cudaError_t launch_fit_mixed(const MixedArgs& a, int block, cudaStream_t s, LaunchTimer* tm = nullptr);
// Persistent work-stealing schedule: per-set channel lists, then per set the
// FP32 search (block threads, `lanes` lanes per channel), judge and repair.
cudaError_t launch_fit_mixed_persistent(const MixedArgs& a, int block, int lanes, cudaStream_t s,
                                        LaunchTimer* tm = nullptr);



// Synthetic generator (synth.cu).
int synth_conditions(int kind, mf_conditions* cond, double* sigma);

// Host-side conversion of a public condition set.
int make_dev_conditions(const mf_conditions& c, DevConditions* d);

void set_last_error(const char* what, cudaError_t e);

}  // namespace mfgb
