/* C++ drop-in for the reference's per-channel fitter over the C ABI of
 * multifit_gb300.h (header-only; link libmultifit_gb300.so).
 *
 *   mfgb::PulseChiSqSNNLS   same member functions as the reference class
 *                           (multifit_cpu/interface/PulseChiSqSNNLS.h:9-59):
 *                           DoFit(samples, samplecor, pederr, bxs, fullpulse,
 *                           fullpulsecov), X(), Errors(), BXs(), ChiSq(),
 *                           disableErrorCalculation(). Each DoFit is a batch of
 *                           one channel through mf_fit_host: source-compatible,
 *                           synchronous, and as slow as one GPU round trip.
 *   mfgb::BatchFitter       the throughput path: queue the channels that share
 *                           a condition set (DoFit's arguments other than the
 *                           samples and pederr), fit them in one mf_fit_host
 *                           call, read X/ChiSq/status per channel.
 *
 * DoFit is a template so that the reference's Eigen types pass straight in
 * (SampleVector, SampleMatrix, BXVector, FullSampleVector, FullSampleMatrix,
 * multifit_cpu/interface/EigenMatrixTypes.h:6-14) without this header
 * including Eigen: any vector with rows() and operator()(i), any matrix with
 * operator()(i, j), will do. */
#ifndef MULTIFIT_GB300_HPP
#define MULTIFIT_GB300_HPP

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "multifit_gb300.h"

namespace mfgb {

/* Fixed-capacity vector standing in for the reference's dynamic Eigen
 * vectors (PulseVector, BXVector: at most 10 entries). */
template <typename T>
class SmallVector {
 public:
  int rows() const { return n_; }
  int size() const { return n_; }
  T coeff(int i) const { return v_[i]; }
  const T& operator()(int i) const { return v_[i]; }
  const T& operator[](int i) const { return v_[i]; }
  T& operator[](int i) { return v_[i]; }
  void resize(int n) {
    n_ = n;
    for (int i = 0; i < MF_MAX_PULSES; ++i) v_[i] = T(0);
  }

 private:
  T v_[MF_MAX_PULSES] = {};
  int n_ = 0;
};
typedef SmallVector<double> PulseVector;
typedef SmallVector<signed char> BXVector;  // signed on every target (plain char is unsigned on Arm)

class Error : public std::runtime_error {
 public:
  Error(const std::string& what, int rc)
      : std::runtime_error(what + ": " + mf_rc_string(rc) + " " + mf_last_error()), rc(rc) {}
  int rc;
};

inline void check(int rc, const char* what) {
  if (rc != MF_OK) throw Error(what, rc);
}

/* One engine context per device, shared by the fitters of a thread. */
class Context {
 public:
  explicit Context(int device = 0) {
    mf_context* c = nullptr;
    check(mf_create(&c, device), "mf_create");
    ctx_.reset(c);
  }
  mf_context* get() const { return ctx_.get(); }

  /* Installs the condition set of DoFit's arguments as set 0, unless it is
   * the one installed last (the tables are built once per distinct set). */
  template <class SM, class BV, class FV, class FM>
  void use(const SM& samplecor, const BV& bxs, const FV& fullpulse, const FM& fullpulsecov) {
    mf_conditions c;
    std::memset(&c, 0, sizeof(c));
    const int N = MF_MAX_SAMPLES, K = int(bxs.rows());
    if (K < 1 || K > MF_MAX_PULSES) throw Error("DoFit: bxs.rows() out of range", MF_EINVAL);
    c.nsamples = N;
    c.npulses = K;
    double fp[MF_FULLPULSE_MAX];
    int8_t bx[MF_MAX_PULSES];
    for (int i = 0; i < MF_FULLPULSE_MAX; ++i) fp[i] = fullpulse(i);
    for (int k = 0; k < K; ++k) bx[k] = static_cast<int8_t>(bxs(k));
    check(mf_build_pulse_matrix(fp, bx, N, K, c.pulse_matrix), "mf_build_pulse_matrix");
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) c.noise_cor[j * N + i] = samplecor(i, j);
    for (int k = 0; k < K; ++k) c.bxs[k] = bx[k];
    bool any = false;
    for (int j = 0; j < MF_FULLPULSE_MAX; ++j)
      for (int i = 0; i < MF_FULLPULSE_MAX; ++i) {
        const double v = fullpulsecov(i, j);
        c.fullpulsecov[j * MF_FULLPULSE_MAX + i] = v;
        any = any || v != 0.;
      }
    c.has_fullpulsecov = any ? 1 : 0;
    if (!any) std::memset(c.fullpulsecov, 0, sizeof(c.fullpulsecov));
    if (have_ && std::memcmp(&c, &last_, sizeof(c)) == 0) return;
    check(mf_set_conditions(ctx_.get(), 0, &c), "mf_set_conditions");
    last_ = c;
    have_ = true;
  }

 private:
  struct Deleter {
    void operator()(mf_context* c) const { mf_destroy(c); }
  };
  std::unique_ptr<mf_context, Deleter> ctx_;
  mf_conditions last_;
  bool have_ = false;
};

/* The reference's PulseChiSqSNNLS, one channel per DoFit. */
class PulseChiSqSNNLS {
 public:
  explicit PulseChiSqSNNLS(std::shared_ptr<Context> ctx = nullptr)
      : ctx_(ctx ? std::move(ctx) : std::make_shared<Context>(0)) {
    mf_default_options(&opt_);  // max_iter 10, eps 1e-11, reference start: multifit_cpu
  }

  /* multifit_cpu/src/PulseChiSqSNNLS.cpp:21-147. Returns false only for input
   * the engine rejects (the reference's DoFit returns true in every case it
   * handles). */
  template <class SV, class SM, class BV, class FV, class FM>
  bool DoFit(const SV& samples, const SM& samplecor, double pederr, const BV& bxs, const FV& fullpulse,
             const FM& fullpulsecov) {
    ctx_->use(samplecor, bxs, fullpulse, fullpulsecov);
    const int K = int(bxs.rows());
    double s[MF_MAX_SAMPLES], amp[MF_MAX_PULSES], chi2 = 0., err = 0.;
    for (int i = 0; i < MF_MAX_SAMPLES; ++i) s[i] = samples(i);
    uint8_t status = 0;
    mf_batch b;
    std::memset(&b, 0, sizeof(b));
    b.n = 1;
    b.sample_stride = MF_MAX_SAMPLES;
    b.amp_stride = MF_MAX_PULSES;
    b.samples = s;
    b.pederr = &pederr;
    b.amplitudes = amp;
    b.chi2 = &chi2;
    b.errors = compute_errors_ ? &err : nullptr;
    b.status = &status;
    opt_.compute_errors = compute_errors_ ? 1 : 0;
    check(mf_fit_host(ctx_->get(), &b, &opt_), "mf_fit_host");
    x_.resize(K);
    errors_.resize(K);
    bxs_.resize(K);
    int intime = -1;  // the first pulse with bx == 0 (PulseChiSqSNNLS.cpp:79-85)
    for (int k = 0; k < K; ++k) {
      x_[k] = amp[k];
      bxs_[k] = static_cast<signed char>(bxs(k));
      if (intime < 0 && bxs(k) == 0) intime = k;
    }
    if (compute_errors_ && intime >= 0) errors_[intime] = err;  // its MINOS-like uncertainty
    chisq_ = chi2;
    return !(status & MF_CH_BADINPUT);
  }

  const PulseVector& X() const { return x_; }
  const PulseVector& Errors() const { return errors_; }
  const BXVector& BXs() const { return bxs_; }
  double ChiSq() const { return chisq_; }
  void disableErrorCalculation() { compute_errors_ = false; }
  /* Engine options beyond the reference's (precision, start mode, max_iter). */
  mf_options& options() { return opt_; }

 private:
  std::shared_ptr<Context> ctx_;
  mf_options opt_;
  PulseVector x_, errors_;
  BXVector bxs_;
  double chisq_ = 0.;
  bool compute_errors_ = true;  // the reference's default (PulseChiSqSNNLS.cpp:14)
};

/* Many channels of one condition set in one call (the doFitWrapper shape of
 * multifit_gpu/interface/PulseChiSqSNNLSWrapper.h:11, without per-call device
 * allocation). */
class BatchFitter {
 public:
  explicit BatchFitter(std::shared_ptr<Context> ctx = nullptr)
      : ctx_(ctx ? std::move(ctx) : std::make_shared<Context>(0)) {
    mf_default_options(&opt_);
  }
  template <class SM, class BV, class FV, class FM>
  void conditions(const SM& samplecor, const BV& bxs, const FV& fullpulse, const FM& fullpulsecov) {
    ctx_->use(samplecor, bxs, fullpulse, fullpulsecov);
    K_ = int(bxs.rows());
  }
  template <class SV>
  void add(const SV& samples, double pederr) {
    for (int i = 0; i < MF_MAX_SAMPLES; ++i) samples_.push_back(samples(i));
    pederr_.push_back(pederr);
  }
  std::size_t size() const { return pederr_.size(); }
  /* Fits every queued channel (synchronous). */
  void run() {
    const int64_t n = int64_t(pederr_.size());
    amp_.assign(size_t(n) * MF_MAX_PULSES, 0.);
    chi2_.assign(size_t(n), 0.);
    status_.assign(size_t(n), 0);
    mask_.assign(size_t(n), 0);
    if (n == 0) return;
    mf_batch b;
    std::memset(&b, 0, sizeof(b));
    b.n = n;
    b.sample_stride = MF_MAX_SAMPLES;
    b.amp_stride = MF_MAX_PULSES;
    b.samples = samples_.data();
    b.pederr = pederr_.data();
    b.amplitudes = amp_.data();
    b.chi2 = chi2_.data();
    b.active_mask = mask_.data();
    b.status = status_.data();
    check(mf_fit_host(ctx_->get(), &b, &opt_), "mf_fit_host");
  }
  void clear() {
    samples_.clear();
    pederr_.clear();
  }
  const double* X(std::size_t i) const { return amp_.data() + i * MF_MAX_PULSES; }
  double ChiSq(std::size_t i) const { return chi2_[i]; }
  uint8_t status(std::size_t i) const { return status_[i]; }
  uint16_t active_mask(std::size_t i) const { return mask_[i]; }
  int npulses() const { return K_; }
  mf_options& options() { return opt_; }

 private:
  std::shared_ptr<Context> ctx_;
  mf_options opt_;
  int K_ = 0;
  std::vector<double> samples_, pederr_, amp_, chi2_;
  std::vector<uint8_t> status_;
  std::vector<uint16_t> mask_;
};

}  // namespace mfgb

#endif /* MULTIFIT_GB300_HPP */
