// Host code under AddressSanitizer and UndefinedBehaviorSanitizer, run by
// tests/test_sanitize_host.py on the CPU (built with -fsanitize=address,
// undefined -fno-sanitize-recover=all, so any finding aborts the process).
//
//   sanitize_host oracle
//       the oracle (oracle/multifit_oracle.cpp, linked in) over every shape
//       N, K in 1..10, both FNNLS variants and starts, max_iter 1/10/1000,
//       MINOS errors and a pulse covariance, and edge channels: NaN and Inf
//       samples, zero / negative / NaN pederr, all-zero samples, amplitudes
//       of 1e12, a covariance that is not positive definite.
//   sanitize_host inflate <streams.bin>
//       the zlib decoder on the streams (as rootio_check inflate), then on
//       every stream with random bytes flipped: each call must return or throw
//       FormatError.
//   sanitize_host rootio-fuzz <file> <mutations> <seed>
//       the ROOT-format reader on copies of the file with 1-8 random bytes
//       changed: opening, listing, reading the Samples tree's branches must
//       return or throw FormatError.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <limits>
#include <string>
#include <vector>

#include "multifit_gb300_io.hpp"

extern "C" {
int oracle_fit_batch(int64_t n, int N, int K, const double* samples, int sample_stride, const double* pederr,
                     const double* P, const double* R, const double* fpc, const int8_t* bxs, double eps,
                     int max_iter_nnls, int max_iter_outer, double dchi2_tol, int variant, int start,
                     int compute_errors, int nthreads, double* amplitudes, double* chi2, uint16_t* mask,
                     uint8_t* status, int32_t* iters, double* err, double* flops);
double oracle_nnls_bruteforce(const double* A, const double* b, int N, int K, double* x_out);
int oracle_nnls_lawson_hanson(const double* A, const double* b, int N, int K, double* x, int max_iter);
}

namespace {

struct Lcg {  // 64-bit linear congruential generator (Knuth's MMIX constants)
  uint64_t s;
  explicit Lcg(uint64_t seed) : s(seed * 2 + 1) {}
  uint64_t next() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return s >> 11;
  }
  double uniform() { return double(next()) * 0x1.0p-53; }
  double normal() {  // Box-Muller
    const double u = std::max(uniform(), 1e-300), v = uniform();
    return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
  }
};

int run_oracle() {
  Lcg rng(11);
  const double nan = std::numeric_limits<double>::quiet_NaN(), inf = std::numeric_limits<double>::infinity();
  int fits = 0;
  for (int N = 1; N <= 10; ++N) {
    for (int K = 1; K <= N; ++K) {
      // CRRC-like columns, each starting one sample later (column-major)
      std::vector<double> P(size_t(N * K), 0.0), R(static_cast<size_t>(N * N)), fpc(size_t((N + 9) * (N + 9)), 0.0);
      for (int k = 0; k < K; ++k)
        for (int i = k; i < N; ++i) {
          const double t = double(i - k + 1);
          P[size_t(k * N + i)] = t * t * std::exp(-t / 2.0) / (16.0 * std::exp(-2.0));
        }
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) R[size_t(j * N + i)] = std::pow(0.7, std::abs(i - j));
      for (int i = 0; i < N + 9; ++i) fpc[size_t(i * (N + 9) + i)] = 1e-4;
      std::vector<int8_t> bxs(static_cast<size_t>(K));
      for (int k = 0; k < K; ++k) bxs[size_t(k)] = int8_t(k - K / 2);
      const int n = 16;
      std::vector<double> s(static_cast<size_t>(n * N)), ped(static_cast<size_t>(n), 0.05);
      for (int c = 0; c < n; ++c) {
        std::vector<double> a(static_cast<size_t>(K));
        for (int k = 0; k < K; ++k) a[size_t(k)] = rng.uniform() < 0.5 ? 0.0 : 100.0 * rng.uniform();
        for (int i = 0; i < N; ++i) {
          double v = 0.05 * rng.normal();
          for (int k = 0; k < K; ++k) v += P[size_t(k * N + i)] * a[size_t(k)];
          s[size_t(c * N + i)] = v;
        }
      }
      // edge channels
      s[0] = nan;
      s[size_t(1 * N)] = inf;
      ped[2] = 0.0;
      ped[3] = -1.0;
      ped[4] = nan;
      for (int i = 0; i < N; ++i) s[size_t(5 * N + i)] = 0.0;
      for (int i = 0; i < N; ++i) s[size_t(6 * N + i)] *= 1e10;
      std::vector<double> amp(static_cast<size_t>(n * K)), chi2(static_cast<size_t>(n)), err(static_cast<size_t>(n)), flops(static_cast<size_t>(n));
      std::vector<uint16_t> mask(static_cast<size_t>(n));
      std::vector<uint8_t> status(static_cast<size_t>(n));
      std::vector<int32_t> iters(static_cast<size_t>(n * 3));
      for (int variant = 0; variant < 2; ++variant)
        for (int start = 0; start < 2; ++start)
          for (int max_iter : {1, 10, 1000})
            for (int extras = 0; extras < 2; ++extras) {
              const int rc = oracle_fit_batch(n, N, K, s.data(), N, ped.data(), P.data(), R.data(),
                                              extras ? fpc.data() : nullptr, bxs.data(), 1e-11, max_iter, 50, 1e-3,
                                              variant, start, extras, 1, amp.data(), chi2.data(), mask.data(),
                                              status.data(), iters.data(), err.data(), flops.data());
              if (rc != 0) return 1;
              ++fits;
            }
      // a correlation matrix that is not positive definite
      std::vector<double> Rbad(R);
      for (int i = 0; i + 1 < N; ++i) Rbad[size_t(i * N + i + 1)] = Rbad[size_t((i + 1) * N + i)] = 1.5;
      if (oracle_fit_batch(n, N, K, s.data(), N, ped.data(), P.data(), Rbad.data(), nullptr, bxs.data(), 1e-11, 10,
                           50, 1e-3, 1, 0, 0, 1, amp.data(), chi2.data(), mask.data(), status.data(), iters.data(),
                           err.data(), nullptr) != 0)
        return 1;
      // the independent solvers on the whitened-free problem A = P, b = first samples
      std::vector<double> x(static_cast<size_t>(K));
      oracle_nnls_bruteforce(P.data(), &s[size_t(7 * N)], N, K, x.data());
      oracle_nnls_lawson_hanson(P.data(), &s[size_t(7 * N)], N, K, x.data(), 100);
      fits += 2;
    }
  }
  std::printf("ok %d\n", fits);
  return 0;
}

std::vector<uint8_t> read_all(const char* path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

int run_inflate(const char* path) {
  const std::vector<uint8_t> d = read_all(path);
  Lcg rng(5);
  size_t p = 0;
  int ok = 0, rejected = 0;
  while (p + 16 <= d.size()) {
    uint64_t raw = 0, comp = 0;
    std::memcpy(&raw, &d[p], 8);
    std::memcpy(&comp, &d[p + 8], 8);
    p += 16;
    std::vector<uint8_t> z(d.begin() + long(p), d.begin() + long(p + comp));
    const std::vector<uint8_t> got = mfgb::rootio::detail::zlib_inflate(z.data(), z.size(), raw);
    if (got.size() != raw || (raw && std::memcmp(got.data(), &d[p + comp], raw) != 0)) return 1;
    ++ok;
    for (int m = 0; m < 4 && !z.empty(); ++m) {
      std::vector<uint8_t> bad(z);
      const int flips = 1 + int(rng.next() % 4);
      for (int f = 0; f < flips; ++f) bad[size_t(rng.next() % bad.size())] ^= uint8_t(1 + rng.next() % 255);
      if (rng.next() % 4 == 0) bad.resize(size_t(rng.next() % bad.size()));  // truncated too
      try {
        mfgb::rootio::detail::zlib_inflate(bad.data(), bad.size(), raw);
      } catch (const mfgb::rootio::FormatError&) {
        ++rejected;
      }
    }
    p += comp + raw;
  }
  std::printf("ok %d rejected %d\n", ok, rejected);
  return 0;
}

template <typename F>
void attempt(F&& f, int& ok, int& rejected) {
  try {
    f();
    ++ok;
  } catch (const mfgb::rootio::FormatError&) {
    ++rejected;
  }
}

int run_rootio_fuzz(const char* path, int mutations, uint64_t seed) {
  const std::vector<uint8_t> orig = read_all(path);
  Lcg rng(seed);
  int ok = 0, rejected = 0;
  for (int m = 0; m < mutations; ++m) {
    std::vector<uint8_t> d(orig);
    const int flips = 1 + int(rng.next() % 8);
    for (int f = 0; f < flips; ++f) d[size_t(rng.next() % d.size())] = uint8_t(rng.next());
    attempt(
        [&] {
          const mfgb::rootio::RootFile file(d, "mutated");
          (void)file.walk();
          for (const auto& k : file.keys()) {
            if (k.class_name == "TTree") {
              const mfgb::rootio::Tree t = file.tree(k.name);
              attempt([&] { (void)t.array<double>("amplitudeTruth"); }, ok, rejected);
              attempt([&] { (void)t.vectors<double>("samples"); }, ok, rejected);
            } else if (k.class_name.rfind("TDirectory", 0) == 0) {
              for (const auto& sub : file.keys(k.name)) {
                const std::string path = k.name + "/" + sub.name;
                if (sub.class_name == "TGraph") attempt([&] { (void)file.graph(path); }, ok, rejected);
                if (sub.class_name == "TTree")
                  attempt([&] { (void)file.tree(path).array<float>("timeMin"); }, ok, rejected);
              }
            }
          }
        },
        ok, rejected);
  }
  std::printf("ok %d rejected %d\n", ok, rejected);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "";
  if (mode == "oracle" && argc == 2) return run_oracle();
  if (mode == "inflate" && argc == 3) return run_inflate(argv[2]);
  if (mode == "rootio-fuzz" && argc == 5) return run_rootio_fuzz(argv[2], std::atoi(argv[3]), std::strtoull(argv[4], nullptr, 10));
  std::fprintf(stderr, "usage: sanitize_host oracle | inflate <streams.bin> | rootio-fuzz <file> <n> <seed>\n");
  return 2;
}
