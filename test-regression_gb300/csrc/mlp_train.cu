// Host side of the learned warm start: parameters, training loop on the
// GPU (the project's own forward/backward/Adam kernels of mlp.cu), weight I/O
// and inference launches.
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "mf_internal.h"
#include "mlp.h"
#include "mlp_state.h"

namespace mfgb {

namespace {
typedef __nv_bfloat16 bf16;

inline unsigned blocks(int64_t n, int t) { return unsigned((n + t - 1) / t); }

cudaError_t pack_all(MlpState& s, cudaStream_t st) {
  pack_weights_kernel<<<blocks(MLP_H * MLP_IN, 256), 256, 0, st>>>(s.params + P_W1, s.W1h, nullptr, MLP_H, MLP_IN);
  pack_weights_kernel<<<blocks(MLP_H * MLP_H, 256), 256, 0, st>>>(s.params + P_W2, s.W2h, s.W2t, MLP_H, MLP_H);
  pack_weights_kernel<<<blocks(MLP_OUT * MLP_H, 256), 256, 0, st>>>(s.params + P_W3, s.W3h, s.W3t, MLP_OUT, MLP_H);
  return cudaGetLastError();
}

template <typename T>
cudaError_t alloc(T** p, size_t count) {
  return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
}
}  // namespace

void mlp_free(MlpState& s) {
  void* ps[] = {s.params, s.grads, s.m, s.v, s.W1h, s.W2h, s.W3h, s.W2t, s.W3t, s.warm_mask, s.warm_amp, s.infer_err};
  for (void* p : ps) cudaFree(p);
  s = MlpState();
}

int mlp_init(MlpState& s, int device, int set, uint64_t seed) {
  mlp_free(s);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = alloc(&s.params, P_COUNT);
  if (e == cudaSuccess) e = alloc(&s.grads, P_COUNT);
  if (e == cudaSuccess) e = alloc(&s.m, P_COUNT);
  if (e == cudaSuccess) e = alloc(&s.v, P_COUNT);
  if (e == cudaSuccess) e = alloc(&s.W1h, MLP_H * MLP_IN);
  if (e == cudaSuccess) e = alloc(&s.W2h, MLP_H * MLP_H);
  if (e == cudaSuccess) e = alloc(&s.W3h, MLP_OUT * MLP_H);
  if (e == cudaSuccess) e = alloc(&s.W2t, MLP_H * MLP_H);
  if (e == cudaSuccess) e = alloc(&s.W3t, MLP_OUT * MLP_H);
  if (e == cudaSuccess) e = alloc(&s.warm_mask, MlpState::kChunk);
  if (e == cudaSuccess) e = alloc(&s.warm_amp, MlpState::kChunk * 10);
  if (e == cudaSuccess) e = alloc(&s.infer_err, 1);
  if (e != cudaSuccess) {
    set_last_error("mlp_init cudaMalloc", e);
    mlp_free(s);
    return MF_ENOMEM;
  }
  s.set = set;
  // He-normal weights (std sqrt(2/fan_in)), zero biases; unused outputs stay zero
  std::vector<float> h(P_COUNT, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int i = 0; i < MLP_H * MLP_IN; ++i)
    h[P_W1 + i] = (i % MLP_IN) < 12 ? nd(rng) * std::sqrt(2.f / 12.f) : 0.f;
  for (int i = 0; i < MLP_H * MLP_H; ++i) h[P_W2 + i] = nd(rng) * std::sqrt(2.f / MLP_H);
  for (int i = 0; i < 20 * MLP_H; ++i) h[P_W3 + i] = nd(rng) * std::sqrt(1.f / MLP_H);
  e = cudaMemcpy(s.params, h.data(), sizeof(float) * P_COUNT, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(s.m, 0, sizeof(float) * P_COUNT);
  if (e == cudaSuccess) e = cudaMemset(s.v, 0, sizeof(float) * P_COUNT);
  if (e == cudaSuccess) e = cudaMemset(s.infer_err, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = pack_all(s, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    set_last_error("mlp_init upload", e);
    mlp_free(s);
    return MF_ECUDA;
  }
  s.step = 0;
  s.ready = true;
  return MF_OK;
}

int mlp_set_weights(MlpState& s, const float* host) {
  if (!s.ready) return MF_ENOTRAINED;
  cudaError_t e = cudaMemcpy(s.params, host, sizeof(float) * P_COUNT, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = pack_all(s, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    set_last_error("mlp_set_weights", e);
    return MF_ECUDA;
  }
  s.trained = true;
  return MF_OK;
}

int mlp_get_weights(const MlpState& s, float* host) {
  if (!s.ready) return MF_ENOTRAINED;
  cudaError_t e = cudaMemcpy(host, s.params, sizeof(float) * P_COUNT, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_last_error("mlp_get_weights", e);
    return MF_ECUDA;
  }
  return MF_OK;
}

void fill_infer_args(const MlpState& s, const HostTables& tab, int intime_unused, MlpInferArgs* a) {
  (void)intime_unused;
  std::memset(a, 0, sizeof(*a));
  a->set = s.set;
  std::memcpy(a->W32, tab.W32, sizeof(a->W32));
  for (int k = 0; k < 10; ++k) a->inv_gnorm[k] = tab.gnorm2[k] > 0 ? float(1.0 / std::sqrt(tab.gnorm2[k])) : 0.f;
  a->W1 = s.W1h;
  a->W2 = s.W2h;
  a->W3 = s.W3h;
  a->b1 = s.params + P_B1;
  a->b2 = s.params + P_B2;
  a->b3 = s.params + P_B3;
  a->err = s.infer_err;
  a->test_stall = s.test_stall;
}

// One training run over n channels whose converged amplitudes are given.
int mlp_train(MlpState& s, const HostTables& tab, int64_t n, int sample_stride, const double* samples,
              const double* pederr, const uint8_t* ctype, const double* amps, int amp_stride,
              const mf_mlp_train_params& tp, float* epoch_loss, cudaStream_t st, MlpGradProbe* probe) {
  if (!s.ready) return MF_ENOTRAINED;
  const int B = tp.batch;
  if (B < 64 || B % 64 || n < B) return MF_EINVAL;
  const int64_t nb = n / B;
  bf16 *X = nullptr, *H1 = nullptr, *H2 = nullptr, *dO = nullptr, *dZ2 = nullptr, *dZ1 = nullptr;
  float *scale = nullptr, *T = nullptr, *Z1 = nullptr, *Z2 = nullptr, *O = nullptr, *dH2 = nullptr, *dH1 = nullptr,
        *loss = nullptr, *gnorm = nullptr;
  cudaError_t e = alloc(&X, n * MLP_IN);
  if (e == cudaSuccess) e = alloc(&scale, n);
  if (e == cudaSuccess) e = alloc(&T, n * 20);
  if (e == cudaSuccess) e = alloc(&Z1, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&Z2, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&O, int64_t(B) * MLP_OUT);
  if (e == cudaSuccess) e = alloc(&H1, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&H2, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&dO, int64_t(B) * MLP_OUT);
  if (e == cudaSuccess) e = alloc(&dH2, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&dH1, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&dZ2, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&dZ1, int64_t(B) * MLP_H);
  if (e == cudaSuccess) e = alloc(&loss, tp.epochs > 0 ? tp.epochs : 1);
  if (e == cudaSuccess) e = alloc(&gnorm, 10);
  int rc = MF_OK;
  if (e == cudaSuccess) {
    float g[10];
    for (int k = 0; k < 10; ++k) g[k] = float(std::sqrt(tab.gnorm2[k]));
    e = cudaMemcpyAsync(gnorm, g, sizeof(g), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, sizeof(float) * (tp.epochs > 0 ? tp.epochs : 1), st);
  }
  if (e == cudaSuccess) {
    MlpFeatArgs fa;
    std::memset(&fa, 0, sizeof(fa));
    fa.n = n;
    fa.sample_stride = sample_stride;
    fa.samples = samples;
    fa.pederr = pederr;
    fa.ctype = ctype;
    fa.set = s.set;
    fa.N = tab.N;
    std::memcpy(fa.W32, tab.W32, sizeof(fa.W32));
    fa.X = X;
    fa.scale = scale;
    mlp_features_kernel<<<blocks(n, 256), 256, 0, st>>>(fa);
    mlp_targets_kernel<<<blocks(n, 256), 256, 0, st>>>(n, amps, amp_stride, scale, gnorm, T);
    e = cudaGetLastError();
  }
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const int epochs = probe ? 1 : tp.epochs;
  for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
    for (int64_t bi = 0; bi < nb && e == cudaSuccess; ++bi) {
      const bf16* Xb = X + bi * int64_t(B) * MLP_IN;
      const float* Tb = T + bi * int64_t(B) * 20;
      GemmArgs g;
      // forward
      std::memset(&g, 0, sizeof(g));
      g.err = s.infer_err;
      g.test_stall = s.test_stall;
      g.A = Xb; g.a_si = MLP_IN; g.a_sk = 1;
      g.B = s.W1h; g.b_sj = MLP_IN; g.b_sk = 1;
      g.M = B; g.N = MLP_H; g.K = MLP_IN; g.k_split = MLP_IN;
      g.C = Z1; g.ldc = MLP_H; g.bias = s.params + P_B1; g.H = H1; g.ldh = MLP_H;
      e = launch_gemm(EPI_BIAS_RELU, true, true, g, 1, st);
      g.A = H1; g.a_si = MLP_H; g.B = s.W2h; g.b_sj = MLP_H; g.K = MLP_H; g.k_split = MLP_H;
      g.C = Z2; g.bias = s.params + P_B2; g.H = H2;
      if (e == cudaSuccess) e = launch_gemm(EPI_BIAS_RELU, true, true, g, 1, st);
      g.A = H2; g.B = s.W3h; g.N = MLP_OUT; g.C = O; g.ldc = MLP_OUT; g.bias = s.params + P_B3; g.H = nullptr;
      if (e == cudaSuccess) e = launch_gemm(EPI_BIAS, true, true, g, 1, st);
      if (e != cudaSuccess) break;
      mlp_loss_kernel<<<blocks(B, 256), 256, 0, st>>>(B, O, Tb, tp.amp_weight, dO, loss + ep);
      e = cudaMemsetAsync(s.grads, 0, sizeof(float) * P_COUNT, st);
      // layer 3 gradients
      const int ks = 256, splits = (B + ks - 1) / ks;
      std::memset(&g, 0, sizeof(g));
      g.err = s.infer_err;
      g.test_stall = s.test_stall;
      g.A = dO; g.a_si = 1; g.a_sk = MLP_OUT;
      g.B = H2; g.b_sj = 1; g.b_sk = MLP_H;
      g.M = MLP_OUT; g.N = MLP_H; g.K = B; g.k_split = ks; g.C = s.grads + P_W3; g.ldc = MLP_H;
      if (e == cudaSuccess) e = launch_gemm(EPI_ATOMIC, false, false, g, splits, st);
      bias_grad_kernel<<<64, MLP_OUT, 0, st>>>(B, MLP_OUT, dO, s.grads + P_B3);
      std::memset(&g, 0, sizeof(g));
      g.err = s.infer_err;
      g.test_stall = s.test_stall;
      g.A = dO; g.a_si = MLP_OUT; g.a_sk = 1;
      g.B = s.W3t; g.b_sj = MLP_OUT; g.b_sk = 1;
      g.M = B; g.N = MLP_H; g.K = MLP_OUT; g.k_split = MLP_OUT; g.C = dH2; g.ldc = MLP_H;
      if (e == cudaSuccess) e = launch_gemm(EPI_STORE, true, true, g, 1, st);
      relu_backward_kernel<<<blocks(int64_t(B) * MLP_H, 256), 256, 0, st>>>(int64_t(B) * MLP_H, dH2, Z2, dZ2);
      // layer 2 gradients
      std::memset(&g, 0, sizeof(g));
      g.err = s.infer_err;
      g.test_stall = s.test_stall;
      g.A = dZ2; g.a_si = 1; g.a_sk = MLP_H;
      g.B = H1; g.b_sj = 1; g.b_sk = MLP_H;
      g.M = MLP_H; g.N = MLP_H; g.K = B; g.k_split = ks; g.C = s.grads + P_W2; g.ldc = MLP_H;
      if (e == cudaSuccess) e = launch_gemm(EPI_ATOMIC, false, false, g, splits, st);
      bias_grad_kernel<<<64, MLP_H, 0, st>>>(B, MLP_H, dZ2, s.grads + P_B2);
      std::memset(&g, 0, sizeof(g));
      g.err = s.infer_err;
      g.test_stall = s.test_stall;
      g.A = dZ2; g.a_si = MLP_H; g.a_sk = 1;
      g.B = s.W2t; g.b_sj = MLP_H; g.b_sk = 1;
      g.M = B; g.N = MLP_H; g.K = MLP_H; g.k_split = MLP_H; g.C = dH1; g.ldc = MLP_H;
      if (e == cudaSuccess) e = launch_gemm(EPI_STORE, true, true, g, 1, st);
      relu_backward_kernel<<<blocks(int64_t(B) * MLP_H, 256), 256, 0, st>>>(int64_t(B) * MLP_H, dH1, Z1, dZ1);
      // layer 1 gradients
      std::memset(&g, 0, sizeof(g));
      g.err = s.infer_err;
      g.test_stall = s.test_stall;
      g.A = dZ1; g.a_si = 1; g.a_sk = MLP_H;
      g.B = Xb; g.b_sj = 1; g.b_sk = MLP_IN;
      g.M = MLP_H; g.N = MLP_IN; g.K = B; g.k_split = ks; g.C = s.grads + P_W1; g.ldc = MLP_IN;
      if (e == cudaSuccess) e = launch_gemm(EPI_ATOMIC, false, false, g, splits, st);
      bias_grad_kernel<<<64, MLP_H, 0, st>>>(B, MLP_H, dZ1, s.grads + P_B1);
      if (probe) {  // gradient check: one forward/backward, no update
        float* Xf = nullptr;
        if (e == cudaSuccess) e = cudaMemcpyAsync(probe->grads, s.grads, sizeof(float) * P_COUNT, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(probe->targets, T, sizeof(float) * B * 20, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(probe->features, X, sizeof(bf16) * B * MLP_IN, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(probe->loss, loss, sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        (void)Xf;
        break;
      }
      // Adam and the bf16 copies
      ++s.step;
      const float c1 = 1.f - std::pow(b1, float(s.step)), c2 = 1.f - std::pow(b2, float(s.step));
      adam_kernel<<<blocks(P_COUNT, 256), 256, 0, st>>>(P_COUNT, s.params, s.grads, s.m, s.v, tp.lr, b1, b2, eps, c1,
                                                       c2);
      if (e == cudaSuccess) e = pack_all(s, st);
      if (e == cudaSuccess) e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess && !probe && epoch_loss && tp.epochs > 0) {
    e = cudaMemcpyAsync(epoch_loss, loss, sizeof(float) * tp.epochs, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (int ep = 0; ep < tp.epochs; ++ep) epoch_loss[ep] /= float(nb);
  }
  if (e == cudaSuccess) {
    // a bounded tensor-core wait of a training GEMM gave up: its products are
    // missing from the weights, so the network is not trained
    unsigned flags = 0;
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(&flags, s.infer_err, sizeof(flags), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && (flags & MLP_ERR_TRAIN_TIMEOUT)) {
      flags &= ~MLP_ERR_TRAIN_TIMEOUT;
      e = cudaMemcpy(s.infer_err, &flags, sizeof(flags), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) {
        set_last_error("mlp_train: a tensor-core wait of a training GEMM timed out", cudaSuccess);
        rc = MF_ETIMEOUT;
      }
    }
  }
  if (e != cudaSuccess) {
    set_last_error("mlp_train", e);
    rc = MF_ECUDA;
  }
  if (!probe) s.trained = rc == MF_OK;  // a failed training has modified the weights
  cudaStreamSynchronize(st);
  void* ps[] = {X, H1, H2, dO, dZ2, dZ1, scale, T, Z1, Z2, O, dH2, dH1, loss, gnorm};
  for (void* p : ps) cudaFree(p);
  return rc;
}

}  // namespace mfgb
