// MLP state owned by a context (learned warm start).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "mf_internal.h"
#include "mlp.h"

namespace mfgb {

// Flat FP32 parameter layout: W1 [128][16] | b1 [128] | W2 [128][128] | b2 [128] | W3 [32][128] | b3 [32]
constexpr int P_W1 = 0;
constexpr int P_B1 = P_W1 + MLP_H * MLP_IN;
constexpr int P_W2 = P_B1 + MLP_H;
constexpr int P_B2 = P_W2 + MLP_H * MLP_H;
constexpr int P_W3 = P_B2 + MLP_H;
constexpr int P_B3 = P_W3 + MLP_OUT * MLP_H;
constexpr int P_COUNT = P_B3 + MLP_OUT;

struct MlpState {
  bool ready = false, trained = false;
  int set = 0;
  int step = 0;
  float* params = nullptr;
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  __nv_bfloat16* W1h = nullptr;
  __nv_bfloat16* W2h = nullptr;
  __nv_bfloat16* W3h = nullptr;
  __nv_bfloat16* W2t = nullptr;
  __nv_bfloat16* W3t = nullptr;
  // predictions of one chunk of a warm fit (allocated with the network, so a
  // warm fit allocates nothing)
  static constexpr int64_t kChunk = MIXED_CHUNK;
  uint16_t* warm_mask = nullptr;
  float* warm_amp = nullptr;
  unsigned* infer_err = nullptr;  // inference error word (MLP_ERR_* bits)
  int test_stall = 0;             // mf_mlp_test_stall
};

// Host buffers of a gradient check (one forward/backward on the first batch).
struct MlpGradProbe {
  float* grads;            // [P_COUNT]
  __nv_bfloat16* features; // [batch][MLP_IN] (bit pattern of the bf16 inputs)
  float* targets;          // [batch][20]
  float* loss;             // [1]
};

void mlp_free(MlpState& s);
int mlp_init(MlpState& s, int device, int set, uint64_t seed);
int mlp_set_weights(MlpState& s, const float* host);
int mlp_get_weights(const MlpState& s, float* host);
void fill_infer_args(const MlpState& s, const HostTables& tab, int unused, MlpInferArgs* a);
int mlp_train(MlpState& s, const HostTables& tab, int64_t n, int sample_stride, const double* samples,
              const double* pederr, const uint8_t* ctype, const double* amps, int amp_stride,
              const mf_mlp_train_params& tp, float* epoch_loss, cudaStream_t st, MlpGradProbe* probe = nullptr);

}  // namespace mfgb
