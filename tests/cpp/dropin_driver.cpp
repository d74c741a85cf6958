// The reference driver's per-channel loop (multifit_cpu/src/multifit.cpp:
// 196-227) with the engine's drop-in class in place of the reference's
// PulseChiSqSNNLS. Small array types stand in for the Eigen types of
// multifit_cpu/interface/EigenMatrixTypes.h (Eigen is not needed).
//
// Usage: dropin_driver <in.bin> <out.bin> <batch:0|1>
//   in.bin:  int64 n; double samplecor[10][10] (row i, column j);
//            int8 bxs[10]; double fullpulse[19]; double fullpulsecov[19][19];
//            then n x (double samples[10], double pederr)
//   out.bin: n x (double chi2, double ampl, int32 status, double x[10])
// batch 0: one DoFit per channel; 1: mfgb::BatchFitter over all channels.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "multifit_gb300.hpp"

template <int R>
struct Vec {
  double v[R];
  int rows() const { return R; }
  double operator()(int i) const { return v[i]; }
};
template <int R>
struct Mat {
  double v[R][R];
  double operator()(int i, int j) const { return v[i][j]; }
};
struct BX {
  signed char v[10];
  int rows() const { return 10; }
  signed char operator()(int i) const { return v[i]; }
  signed char coeff(int i) const { return v[i]; }
};

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  long long n = 0;
  Mat<10> samplecor;
  BX bxs;
  Vec<19> fullpulse;
  Mat<19> fullpulsecov;
  bool ok = std::fread(&n, 8, 1, f) == 1 && std::fread(samplecor.v, 8, 100, f) == 100 &&
            std::fread(bxs.v, 1, 10, f) == 10 && std::fread(fullpulse.v, 8, 19, f) == 19 &&
            std::fread(fullpulsecov.v, 8, 361, f) == 361;
  std::vector<Vec<10>> samples(static_cast<size_t>(n));
  std::vector<double> pederr(static_cast<size_t>(n));
  for (long long c = 0; ok && c < n; ++c)
    ok = std::fread(samples[c].v, 8, 10, f) == 10 && std::fread(&pederr[c], 8, 1, f) == 1;
  std::fclose(f);
  if (!ok) return 2;
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  try {
    auto ctx = std::make_shared<mfgb::Context>(0);
    if (std::atoi(argv[3]) == 0) {
      for (long long c = 0; c < n; ++c) {
        mfgb::PulseChiSqSNNLS func(ctx);
        func.disableErrorCalculation();
        const bool status = func.DoFit(samples[c], samplecor, pederr[c], bxs, fullpulse, fullpulsecov);
        const double chi2 = func.ChiSq();
        unsigned ip_in_time = 0;
        for (int ip = 0; ip < func.BXs().rows(); ++ip)
          if (func.BXs().coeff(ip) == 0) {
            ip_in_time = unsigned(ip);
            break;
          }
        const double ampl = status ? func.X()[int(ip_in_time)] : 0.;
        double x[10] = {};
        for (int ip = 0; ip < func.BXs().rows(); ++ip) {
          const int slot = int(func.BXs().coeff(ip)) + 5;
          if (slot >= 0 && slot < 10) x[slot] = func.X()[ip];
        }
        const int st = status ? 1 : 0;
        std::fwrite(&chi2, 8, 1, o);
        std::fwrite(&ampl, 8, 1, o);
        std::fwrite(&st, 4, 1, o);
        std::fwrite(x, 8, 10, o);
      }
    } else {
      mfgb::BatchFitter fit(ctx);
      fit.conditions(samplecor, bxs, fullpulse, fullpulsecov);
      for (long long c = 0; c < n; ++c) fit.add(samples[c], pederr[c]);
      fit.run();
      for (long long c = 0; c < n; ++c) {
        const double chi2 = fit.ChiSq(size_t(c));
        const int st = (fit.status(size_t(c)) & MF_CH_BADINPUT) ? 0 : 1;
        double x[10] = {};
        for (int ip = 0; ip < 10; ++ip) {
          const int slot = int(bxs.v[ip]) + 5;
          if (slot >= 0 && slot < 10) x[slot] = fit.X(size_t(c))[ip];
        }
        const double ampl = st ? x[5] : 0.;
        std::fwrite(&chi2, 8, 1, o);
        std::fwrite(&ampl, 8, 1, o);
        std::fwrite(&st, 4, 1, o);
        std::fwrite(x, 8, 10, o);
      }
    }
  } catch (const mfgb::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    std::fclose(o);
    return 1;
  }
  std::fclose(o);
  return 0;
}
