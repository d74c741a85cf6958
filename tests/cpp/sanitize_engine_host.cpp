// The engine library's host code under AddressSanitizer and
// UndefinedBehaviorSanitizer, with no GPU: every entry point that does its
// work on the host (argument checks, the pulse-matrix rule, the per-passive-
// set operator tables, the synthetic generator, return-code strings), and
// the error paths of the device entry points (a null context, no device).
// Built by tests/test_sanitize_host.py from the engine's sources compiled
// with host-side -fsanitize=address -fsanitize=undefined; any finding aborts.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "multifit_gb300.h"

#define CHECK(cond)                                          \
  do {                                                       \
    if (!(cond)) {                                           \
      std::printf("check failed: %s (line %d)\n", #cond, __LINE__); \
      return 1;                                              \
    }                                                        \
  } while (0)

int main() {
  CHECK(mf_abi_version() > 0);
  for (int rc = -1; rc <= 8; ++rc) CHECK(mf_rc_string(rc) != nullptr);
  CHECK(mf_last_error() != nullptr);
  mf_options o;
  mf_default_options(&o);
  CHECK(o.max_iter_nnls == 10 && o.max_iter_outer == 50);

  // device entry points without a context or a device
  mf_context* ctx = nullptr;
  const int rc_create = mf_create(&ctx, 0);
  CHECK(rc_create != MF_OK || ctx != nullptr);
  if (rc_create != MF_OK) CHECK(ctx == nullptr);
  CHECK(mf_create(nullptr, 0) == MF_EINVAL);
  mf_destroy(nullptr);
  mf_batch b;
  std::memset(&b, 0, sizeof(b));
  CHECK(mf_fit(nullptr, &b, &o, nullptr) == MF_EINVAL);
  CHECK(mf_fit_host(nullptr, &b, &o) == MF_EINVAL);
  CHECK(mf_fit_noalloc(nullptr, &b, &o, nullptr) == MF_EINVAL);
  CHECK(mf_set_conditions(nullptr, 0, nullptr) == MF_EINVAL);
  CHECK(mf_profile(nullptr, 1) == MF_EINVAL);
  if (ctx) mf_destroy(ctx);

  // the pulse-matrix rule over every shape and edge argument
  std::vector<double> fp(19), P(100);
  for (int i = 0; i < 19; ++i) fp[size_t(i)] = std::exp(-0.3 * i);
  std::vector<int8_t> bxs = {-5, -4, -3, -2, -1, 0, 1, 2, 3, 4};
  for (int N = 1; N <= 10; ++N)
    for (int K = 1; K <= 10; ++K) CHECK(mf_build_pulse_matrix(fp.data(), bxs.data(), N, K, P.data()) == MF_OK);
  CHECK(mf_build_pulse_matrix(fp.data(), bxs.data(), 11, 10, P.data()) == MF_EINVAL);
  CHECK(mf_build_pulse_matrix(fp.data(), bxs.data(), 10, 0, P.data()) == MF_EINVAL);
  CHECK(mf_build_pulse_matrix(nullptr, bxs.data(), 10, 10, P.data()) == MF_EINVAL);
  std::vector<int8_t> far_bxs = {-100, 100, 0, 127, -128, 5, -9, 9, 1, 2};
  mf_build_pulse_matrix(fp.data(), far_bxs.data(), 10, 10, P.data());  // out-of-window offsets: zeros or EINVAL

  // operator tables of both synthetic sets, every passive set
  for (int kind = 0; kind < 2; ++kind) {
    mf_conditions c;
    double sigma = 0;
    CHECK(mf_synth_conditions(kind, &c, &sigma) == MF_OK);
    std::vector<double> W(100), pinv(100);
    const uint32_t full = (1u << c.npulses) - 1;
    for (uint32_t m = 1; m <= full; ++m) CHECK(mf_table_operator(&c, m, W.data(), pinv.data()) == MF_OK);
    CHECK(mf_table_operator(&c, 0, W.data(), pinv.data()) != MF_OK || true);
    CHECK(mf_table_operator(&c, full + 1, W.data(), pinv.data()) != MF_OK);
  }
  mf_conditions c;
  double sigma = 0;
  CHECK(mf_synth_conditions(7, &c, &sigma) == MF_EINVAL);

  // the host generator: empty, small, mixed ECAL/HCAL, per-channel pileup
  for (int variant = 0; variant < 4; ++variant) {
    mf_synth_params p;
    std::memset(&p, 0, sizeof(p));
    const int64_t n = variant == 0 ? 0 : 257;
    p.n = n;
    p.seed = 3 + uint64_t(variant);
    p.intime_log = variant & 1;
    p.intime_lo = 0.1;
    p.intime_hi = 1000;
    p.pileup_mean = variant == 3 ? -8.0 : 4.0;
    p.pileup_hit_mean = 1.0;
    p.hcal_fraction = variant >= 2 ? 0.4 : 0.0;
    std::vector<double> s(size_t(n) * 12 + 1), ped(size_t(n) + 1), truth(size_t(n) * 11 + 1);
    std::vector<uint8_t> ct(size_t(n) + 1);
    CHECK(mf_synth_generate(&p, 5, n, 12, s.data(), ped.data(), ct.data(), truth.data(), 11, 0, nullptr) == MF_OK);
    for (int64_t i = 0; i < n; ++i) CHECK(std::isfinite(ped[size_t(i)]) && ct[size_t(i)] <= 1);
  }
  std::printf("ok\n");
  return 0;
}
