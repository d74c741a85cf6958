// The reference driver's run() (multifit_cpu/src/multifit.cpp:45-81 init,
// 83-271 run, first iteration) in C++ against the engine: the Samples tree
// and the pulse shape read by include/multifit_gb300_io.hpp instead of ROOT,
// the per-channel loop through mfgb::PulseChiSqSNNLS instead of the
// reference's class, and its physics check -- mean and RMS of
// (reconstructed - true) in-time amplitude as the histogram h01 (1000 bins
// over [-5, 5)) reports them.
//
// Usage: replay_driver <Samples file> <pulse-shape file> <entries> <batch:0|1>
//   entries: channels to fit (round-robin over the tree, as GetEntry(ie %
//            GetEntries())); 0 = every entry once.
//   batch 0: one DoFit per channel (the driver's lambda); 1: mfgb::BatchFitter.
// Prints "entries N", "mean M", "rms R", "in_range K" and one line per
// channel "x <ampl> <chi2>" (%.17g).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "multifit_gb300.hpp"
#include "multifit_gb300_io.hpp"

namespace {

template <int R>
struct Vec {
  double v[R] = {};
  int rows() const { return R; }
  double operator()(int i) const { return v[i]; }
};
template <int R>
struct Mat {
  double v[R][R] = {};
  double operator()(int i, int j) const { return v[i][j]; }
};
struct BX {
  signed char v[10];
  int rows() const { return 10; }
  signed char operator()(int i) const { return v[i]; }
  signed char coeff(int i) const { return v[i]; }
};

}  // namespace

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: replay_driver <Samples file> <pulse-shape file> <entries> <batch:0|1>\n");
    return 2;
  }
  try {
    mfgb::ecal_data_io io(argv[1], argv[2]);
    const auto fp = mfgb::driver_fullpulse(io.pulse());
    const auto cor = mfgb::driver_noisecor(io.pulse());
    Vec<19> fullpulse;
    Mat<10> noisecor;
    Mat<19> fullpulsecov;  // zero, as the driver's
    BX bxs;
    for (int i = 0; i < 19; ++i) fullpulse.v[i] = fp[size_t(i)];
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j) noisecor.v[i][j] = cor[size_t(i * 10 + j)];
    for (int k = 0; k < 10; ++k) bxs.v[k] = static_cast<signed char>(mfgb::kIoActiveBxs[size_t(k)]);
    long long n = std::atoll(argv[3]);
    if (n <= 0) n = io.entries();
    const bool batch = std::atoi(argv[4]) != 0;

    std::vector<Vec<10>> samples(static_cast<size_t>(n));
    std::vector<double> truth(static_cast<size_t>(n));
    for (long long ie = 0; ie < n; ++ie) {
      const auto entry = io.get_one_entry();
      for (int i = 0; i < 10; ++i) samples[size_t(ie)].v[i] = entry.first[size_t(i)];
      truth[size_t(ie)] = io.truth()[size_t(ie % io.entries())];
    }
    const double pedrms = mfgb::kIoPedrms;
    std::vector<double> ampl(static_cast<size_t>(n)), chi2(static_cast<size_t>(n));
    auto ctx = std::make_shared<mfgb::Context>(0);
    if (!batch) {
      for (long long ie = 0; ie < n; ++ie) {
        mfgb::PulseChiSqSNNLS func(ctx);
        func.disableErrorCalculation();
        const bool status = func.DoFit(samples[size_t(ie)], noisecor, pedrms, bxs, fullpulse, fullpulsecov);
        unsigned ip_in_time = 0;
        for (int ip = 0; ip < func.BXs().rows(); ++ip)
          if (func.BXs().coeff(ip) == 0) {
            ip_in_time = unsigned(ip);
            break;
          }
        ampl[size_t(ie)] = status ? func.X()[int(ip_in_time)] : 0.;
        chi2[size_t(ie)] = func.ChiSq();
      }
    } else {
      mfgb::BatchFitter fit(ctx);
      fit.conditions(noisecor, bxs, fullpulse, fullpulsecov);
      for (long long ie = 0; ie < n; ++ie) fit.add(samples[size_t(ie)], pedrms);
      fit.run();
      for (long long ie = 0; ie < n; ++ie) {
        ampl[size_t(ie)] = fit.X(size_t(ie))[5];  // BXs -5..4: the in-time column is 5
        chi2[size_t(ie)] = fit.ChiSq(size_t(ie));
      }
    }
    // h01: fills outside [-5, 5) are entries but not in the moments
    double sw = 0, sx = 0, sx2 = 0;
    for (long long ie = 0; ie < n; ++ie) {
      const double d = ampl[size_t(ie)] - truth[size_t(ie)];
      if (d >= -5.0 && d < 5.0) {
        sw += 1;
        sx += d;
        sx2 += d * d;
      }
    }
    const double mean = sw > 0 ? sx / sw : 0.0;
    const double rms = sw > 0 ? std::sqrt(std::fabs(sx2 / sw - mean * mean)) : 0.0;
    std::printf("entries %lld\nmean %.17g\nrms %.17g\nin_range %.0f\n", n, mean, rms, sw);
    for (long long ie = 0; ie < n; ++ie) std::printf("x %.17g %.17g\n", ampl[size_t(ie)], chi2[size_t(ie)]);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
