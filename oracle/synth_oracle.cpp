// Synthetic-channel generator of the oracle. TEST INFRASTRUCTURE ONLY: the
// CPU arms of the benchmark and the tests use it to make the same seeded
// channels the engine's generator makes, without loading the engine library.
//
// What it restates:
//   * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
//     easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies with
//     the published multipliers and Weyl key increments.
//   * The per-channel stream layout of the engine's generator: counter
//     (draw block, channel lo, channel hi, 0x6d66), key (seed lo, seed hi ^
//     tag), four words per block, uniforms from 53 bits in (0, 1).
//   * The channel: set draw, in-time amplitude (uniform or log-uniform),
//     per-channel pileup mean, Poisson hits per out-of-time BX by CDF
//     inversion (capped at 64) with exponential energies, Box-Muller normals,
//     noise sigma * chol(R) z with R_ij = rho^|i-j| (the method of the
//     reference's generator, gen/src/gen_data.cpp:303-320).
//   * The condition sets: the ECAL set as the reference driver builds it
//     (12-sample template with its peak at index 2 placed at fullpulse(7..18),
//     multifit_cpu/src/multifit.cpp:57-67, turned into the pulse matrix by the
//     sliding-window rule of PulseChiSqSNNLS::DoFit,
//     multifit_cpu/src/PulseChiSqSNNLS.cpp:49-62), and the HCAL 8x8 set
//     sampled wherever t >= 0.
// Built with -ffp-contract=off; every operation is written in the order the
// engine's host generator evaluates it, so the two agree bit for bit where
// neither contracts (checked by tests/test_oracle_synth.py).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr int KMAX = 10;
constexpr int NSETS = 2;

struct Ctr {
  uint32_t v[4];
};

inline Ctr philox10(Ctr c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = uint64_t(0xD2511F53u) * c.v[0];
    const uint64_t p1 = uint64_t(0xCD9E8D57u) * c.v[2];
    Ctr n;
    n.v[0] = uint32_t(p1 >> 32) ^ c.v[1] ^ k0;
    n.v[1] = uint32_t(p1);
    n.v[2] = uint32_t(p0 >> 32) ^ c.v[3] ^ k1;
    n.v[3] = uint32_t(p0);
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

class Stream {
 public:
  Stream(uint64_t seed, uint64_t channel, uint32_t tag)
      : k0_(uint32_t(seed)), k1_(uint32_t(seed >> 32) ^ tag), lo_(uint32_t(channel)), hi_(uint32_t(channel >> 32)) {}

  uint32_t word() {
    if (pos_ == 4) {
      Ctr c{{block_++, lo_, hi_, 0x6d66u}};
      out_ = philox10(c, k0_, k1_);
      pos_ = 0;
    }
    return out_.v[pos_++];
  }

  double uniform() {
    const uint64_t a = word();
    const uint64_t b = word();
    const uint64_t bits = ((a << 32) | b) >> 11;
    return (double(bits) + 0.5) * (1.0 / 9007199254740992.0);
  }

 private:
  uint32_t k0_, k1_, lo_, hi_;
  uint32_t block_ = 0;
  Ctr out_{{0, 0, 0, 0}};
  int pos_ = 4;
};

struct Params {
  uint64_t seed;
  int intime_log;
  double lo, hi, pileup_mean, hit_mean, hcal_fraction;
};

struct Set {
  int N, K, intime;
  double P[KMAX * KMAX];  // column-major: P[k * N + i]
  double R[KMAX * KMAX];  // column-major, symmetric
  double L[KMAX * KMAX];  // row-major lower Cholesky factor of R, stride KMAX
  double sigma;
  int8_t bxs[KMAX];
};

// Pulse shape (t/tau)^power e^(-t/tau) scaled to peak 1 at t = power tau.
double shape(double t, double tau, int power) {
  if (t < 0) return 0.;
  const double q = t / tau;
  double qp = 1, norm = 1;
  for (int i = 0; i < power; ++i) qp *= q;
  for (int i = 0; i < power; ++i) norm *= double(power);
  return qp * std::exp(-q) * std::exp(double(power)) / norm;
}

// multifit_cpu/src/PulseChiSqSNNLS.cpp:49-62: column k holds fullpulse(i + 4 - bx_k)
// from sample max(0, bx_k + 3) on, zero above.
void sliding_window(const double* fullpulse, const int8_t* bxs, int N, int K, double* P) {
  for (int k = 0; k < K; ++k) {
    const int first = bxs[k] + 3 > 0 ? bxs[k] + 3 : 0;
    for (int i = 0; i < N; ++i) P[k * N + i] = i >= first ? fullpulse[i + 4 - bxs[k]] : 0.;
  }
}

int make_set(int kind, Set* s) {
  std::memset(s, 0, sizeof(*s));
  int power;
  double tau, rho;
  if (kind == 0) {
    s->N = s->K = 10;
    s->intime = 5;
    power = 4;
    tau = 43.0;
    rho = 0.7;
    s->sigma = 0.044;
  } else if (kind == 1) {
    s->N = s->K = 8;
    s->intime = 3;
    power = 2;
    tau = 10.0;
    rho = 0.3;
    s->sigma = 0.8;
  } else {
    return 1;
  }
  const int N = s->N, K = s->K;
  for (int k = 0; k < K; ++k) s->bxs[k] = int8_t(k - s->intime);
  if (kind == 0) {
    double fullpulse[KMAX + 9] = {0};
    for (int j = 0; j < 12; ++j) fullpulse[7 + j] = shape(power * tau + 25.0 * (j - 2), tau, power);
    sliding_window(fullpulse, s->bxs, N, K, s->P);
  } else {
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < N; ++i) s->P[k * N + i] = shape(power * tau + 25.0 * (i - s->intime - s->bxs[k]), tau, power);
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) s->R[j * N + i] = std::pow(rho, std::abs(i - j));
  // row-oriented Cholesky of R (plain products and sums, diagonal by sqrt)
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j) {
      double v = s->R[j * N + i];
      for (int k = 0; k < j; ++k) v -= s->L[i * KMAX + k] * s->L[j * KMAX + k];
      s->L[i * KMAX + j] = i == j ? std::sqrt(v) : v / s->L[j * KMAX + j];
    }
  return 0;
}

void channel(const Params& p, const Set* sets, int nsets, uint64_t ch, double* samp, int stride, double* ped,
             uint8_t* ct, double* truth, int truth_stride) {
  Stream rng(p.seed, ch, 0x5eed);
  const double ut = rng.uniform();
  const int t = (nsets > 1 && ut < p.hcal_fraction) ? 1 : 0;
  const Set& s = sets[t];
  const int N = s.N, K = s.K;
  const double ua = rng.uniform();
  const double a_in = p.intime_log ? p.lo * std::exp(ua * std::log(p.hi / p.lo)) : p.lo + ua * (p.hi - p.lo);
  const double umu = rng.uniform();
  const double mu = p.pileup_mean >= 0 ? p.pileup_mean : -p.pileup_mean * umu;
  double amp[KMAX];
  for (int k = 0; k < K; ++k) {
    if (k == s.intime) {
      amp[k] = a_in;
      continue;
    }
    const double u = rng.uniform();
    double pk = std::exp(-mu), cdf = pk;
    int hits = 0;
    while (u > cdf && hits < 64) {
      ++hits;
      pk *= mu / hits;
      cdf += pk;
    }
    double e = 0;
    for (int h = 0; h < hits; ++h) e += -p.hit_mean * std::log(rng.uniform());
    amp[k] = e;
  }
  double z[KMAX];
  for (int i = 0; i < N; i += 2) {
    const double u1 = rng.uniform(), u2 = rng.uniform();
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double a = 2.0 * 3.14159265358979323846 * u2;
    z[i] = r * std::cos(a);
    if (i + 1 < N) z[i + 1] = r * std::sin(a);
  }
  for (int i = 0; i < N; ++i) {
    double noise = 0, sig = 0;
    for (int j = 0; j <= i; ++j) noise += s.L[i * KMAX + j] * z[j];
    for (int k = 0; k < K; ++k) sig += s.P[k * N + i] * amp[k];
    samp[i] = sig + s.sigma * noise;
  }
  for (int i = N; i < stride; ++i) samp[i] = 0.;
  *ped = s.sigma;
  if (ct) *ct = uint8_t(t);
  if (truth) {
    for (int k = 0; k < truth_stride; ++k) truth[k] = k < K ? amp[k] : 0.;
  }
}

}  // namespace

extern "C" {

// Condition set `kind` (0 = ECAL 10x10, 1 = HCAL 8x8): P column-major (K*N),
// R column-major (N*N), bxs (K), sigma. Returns 0, or 1 for an unknown kind.
int oracle_synth_conditions(int kind, int* N, int* K, double* P, double* R, int8_t* bxs, double* sigma) {
  Set s;
  if (make_set(kind, &s)) return 1;
  *N = s.N;
  *K = s.K;
  std::memcpy(P, s.P, sizeof(double) * s.N * s.K);
  std::memcpy(R, s.R, sizeof(double) * s.N * s.N);
  std::memcpy(bxs, s.bxs, s.K);
  *sigma = s.sigma;
  return 0;
}

// Channels [first, first + count) of the seeded stream. hcal_fraction > 0
// draws the set per channel (ctype then required). nthreads 0 = all cores.
int oracle_synth_generate(uint64_t seed, int intime_log, double lo, double hi, double pileup_mean, double hit_mean,
                          double hcal_fraction, int64_t first, int64_t count, int stride, double* samples,
                          double* pederr, uint8_t* ctype, double* truth, int truth_stride, int nthreads) {
  const Params p{seed, intime_log, lo, hi, pileup_mean, hit_mean, hcal_fraction};
  Set sets[NSETS];
  const int nsets = hcal_fraction > 0 ? 2 : 1;
  for (int t = 0; t < nsets; ++t) make_set(t, &sets[t]);
  if (count < 0 || first < 0 || !samples || !pederr || stride < sets[0].N) return 1;
  if (nsets > 1 && !ctype) return 1;
  if (truth && truth_stride < KMAX) return 1;
  auto work = [&](int64_t a, int64_t b) {
    for (int64_t i = a; i < b; ++i)
      channel(p, sets, nsets, uint64_t(first + i), samples + i * stride, stride, pederr + i, ctype ? ctype + i : nullptr,
              truth ? truth + i * truth_stride : nullptr, truth_stride);
  };
  int nt = nthreads > 0 ? nthreads : int(std::thread::hardware_concurrency());
  if (nt < 1) nt = 1;
  if (count < 4096) nt = 1;
  if (nt == 1) {
    work(0, count);
    return 0;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (count + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const int64_t a = t * chunk, b = a + chunk < count ? a + chunk : count;
    if (a < b) pool.emplace_back(work, a, b);
  }
  for (auto& th : pool) th.join();
  return 0;
}

}  // extern "C"
