// Synthetic channel generator: seeded, counter-based, identical stream layout
// on host and device.
//
// A channel holds an in-time pulse plus Poisson pileup in every out-of-time
// BX, sampled through the condition set's pulse matrix, plus correlated
// Gaussian noise sigma * chol(R) * z with R_ij = rho^|i-j| (the method of the
// reference's generator, gen/src/gen_data.cpp:303-320).
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "mf_internal.h"
#include "philox.cuh"

namespace mfgb {

namespace {

MF_HD double mf_log(double x) { return log(x); }
MF_HD double mf_exp(double x) { return exp(x); }

MF_HD void mf_sincos_2pi(double u, double* s, double* c) {
#if defined(__CUDA_ARCH__)
  sincospi(2.0 * u, s, c);
#else
  const double a = 2.0 * 3.14159265358979323846 * u;
  *s = std::sin(a);
  *c = std::cos(a);
#endif
}

struct SynthSet {
  DevConditions c[MF_MAX_CTYPES];
  double chol[MF_MAX_CTYPES][KMAX * KMAX];  // row-major lower Cholesky factor of R
  double sigma[MF_MAX_CTYPES];
  int n_sets;
};

MF_HD void synth_channel(const mf_synth_params& p, const SynthSet& S, uint64_t ch, double* samp, int stride,
                         double* ped, uint8_t* ct, double* truth, int truth_stride) {
  ChannelRng rng(p.seed, ch, 0x5eed);
  const double ut = rng.uniform();
  int t = 0;
  if (S.n_sets > 1 && ut < p.hcal_fraction) t = 1;
  const DevConditions& c = S.c[t];
  const int N = c.N, K = c.K;

  const double ua = rng.uniform();
  double a_in;
  if (p.intime_log) a_in = p.intime_lo * mf_exp(ua * mf_log(p.intime_hi / p.intime_lo));
  else a_in = p.intime_lo + ua * (p.intime_hi - p.intime_lo);
  const double umu = rng.uniform();
  const double mu = p.pileup_mean >= 0 ? p.pileup_mean : -p.pileup_mean * umu;

  double amp[KMAX];
  for (int k = 0; k < K; ++k) {
    if (k == c.intime_col) {
      amp[k] = a_in;
      continue;
    }
    // Poisson(mu) by inversion of the CDF (mu <= 8 here; capped at 64 hits).
    const double u = rng.uniform();
    double pk = mf_exp(-mu), cdf = pk;
    int hits = 0;
    while (u > cdf && hits < 64) {
      ++hits;
      pk *= mu / hits;
      cdf += pk;
    }
    double e = 0;
    for (int h = 0; h < hits; ++h) e += -p.pileup_hit_mean * mf_log(rng.uniform());
    amp[k] = e;
  }

  double z[KMAX];
  for (int i = 0; i < N; i += 2) {
    const double u1 = rng.uniform(), u2 = rng.uniform();
    const double r = sqrt(-2.0 * mf_log(u1));
    double s, co;
    mf_sincos_2pi(u2, &s, &co);
    z[i] = r * co;
    if (i + 1 < N) z[i + 1] = r * s;
  }
  const double sg = S.sigma[t];
  for (int i = 0; i < N; ++i) {
    double noise = 0;
    for (int j = 0; j <= i; ++j) noise += S.chol[t][i * KMAX + j] * z[j];
    double sig = 0;
    for (int k = 0; k < K; ++k) sig += c.P[k * N + i] * amp[k];
    samp[i] = sig + sg * noise;
  }
  for (int i = N; i < stride; ++i) samp[i] = 0.;
  *ped = sg;
  if (ct) *ct = uint8_t(t);
  if (truth) {
    for (int k = 0; k < K; ++k) truth[k] = amp[k];
    for (int k = K; k < truth_stride; ++k) truth[k] = 0.;
  }
}

__global__ void synth_kernel(mf_synth_params p, SynthSet S, int64_t first, int64_t count, int stride,
                             double* samples, double* pederr, uint8_t* ctype, double* truth, int truth_stride) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
    synth_channel(p, S, uint64_t(first + i), samples + i * stride, stride, pederr + i, ctype ? ctype + i : nullptr,
                  truth ? truth + i * truth_stride : nullptr, truth_stride);
  }
}

double crrc(double t, double tau, int power) {
  if (t < 0) return 0.;
  const double q = t / tau;
  double qp = 1;
  for (int i = 0; i < power; ++i) qp *= q;
  // normalised so that the peak at t = power * tau is 1
  double norm = 1;
  for (int i = 0; i < power; ++i) norm *= double(power);
  return qp * std::exp(-q) * std::exp(double(power)) / norm;
}

void fill_set(SynthSet& S, const DevConditions* conds, const double* chol, const double* sigma, int n_sets) {
  S.n_sets = n_sets;
  for (int t = 0; t < n_sets; ++t) {
    S.c[t] = conds[t];
    std::memcpy(S.chol[t], chol + t * KMAX * KMAX, sizeof(double) * KMAX * KMAX);
    S.sigma[t] = sigma[t];
  }
}

}  // namespace

int synth_conditions(int kind, mf_conditions* c, double* sigma) {
  if (!c || !sigma) return MF_EINVAL;
  std::memset(c, 0, sizeof(*c));
  int N, K, intime_sample, power;
  double tau, rho, sg;
  if (kind == MF_SYNTH_ECAL) {
    N = K = 10; intime_sample = 5; power = 4; tau = 43.0; rho = 0.7; sg = 0.044;
  } else if (kind == MF_SYNTH_HCAL) {
    N = K = 8; intime_sample = 3; power = 2; tau = 10.0; rho = 0.3; sg = 0.8;
  } else {
    return MF_EINVAL;
  }
  c->nsamples = N;
  c->npulses = K;
  for (int k = 0; k < K; ++k) c->bxs[k] = int8_t(k - intime_sample);  // column k peaks at sample k
  if (kind == MF_SYNTH_ECAL) {
    // As the reference driver: a 12-sample template whose index 2 is the
    // peak, placed at fullpulse(7..18) (multifit_cpu/src/multifit.cpp:57-67),
    // and the sliding-window rule of PulseChiSqSNNLS::DoFit (:49-62), so a
    // pulse starts two samples before its peak.
    double fullpulse[MF_FULLPULSE_MAX] = {0};
    for (int j = 0; j < 12; ++j) fullpulse[7 + j] = crrc(power * tau + 25.0 * (j - 2), tau, power);
    mf_build_pulse_matrix(fullpulse, c->bxs, N, K, c->pulse_matrix);
  } else {
    // HCAL: the pulse sampled wherever t >= 0 (t = 2 tau + 25 ns (i - 3 - bx)).
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < N; ++i) {
        const double t = power * tau + 25.0 * (i - intime_sample - c->bxs[k]);
        c->pulse_matrix[k * N + i] = crrc(t, tau, power);
      }
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) c->noise_cor[j * N + i] = std::pow(rho, std::abs(i - j));
  c->has_fullpulsecov = 0;
  *sigma = sg;
  return MF_OK;
}

static void chol_lower(const DevConditions& c, double* L) {
  const int N = c.N;
  std::memset(L, 0, sizeof(double) * KMAX * KMAX);
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = c.R[j * N + i];
      for (int k = 0; k < j; ++k) s -= L[i * KMAX + k] * L[j * KMAX + k];
      L[i * KMAX + j] = (i == j) ? std::sqrt(s) : s / L[j * KMAX + j];
    }
  }
}

}  // namespace mfgb

using namespace mfgb;

namespace {
int prepare_synth(const mf_synth_params* p, SynthSet* S) {
  if (!p || p->n < 0) return MF_EINVAL;
  mf_conditions c;
  DevConditions d[MF_MAX_CTYPES];
  double chol[MF_MAX_CTYPES * KMAX * KMAX];
  double sigma[MF_MAX_CTYPES];
  const int n_sets = p->hcal_fraction > 0 ? 2 : 1;
  for (int t = 0; t < n_sets; ++t) {
    synth_conditions(t == 0 ? MF_SYNTH_ECAL : MF_SYNTH_HCAL, &c, &sigma[t]);
    make_dev_conditions(c, &d[t]);
    chol_lower(d[t], chol + t * KMAX * KMAX);
  }
  fill_set(*S, d, chol, sigma, n_sets);
  return MF_OK;
}
}  // namespace

extern "C" int mf_synth_conditions(int kind, mf_conditions* cond, double* sigma) {
  return synth_conditions(kind, cond, sigma);
}

extern "C" int mf_synth_generate(const mf_synth_params* p, int64_t first, int64_t count, int sample_stride,
                                 double* samples, double* pederr, uint8_t* ctype, double* truth, int truth_stride,
                                 int on_device, void* stream) {
  SynthSet S;
  int rc = prepare_synth(p, &S);
  if (rc) return rc;
  if (count < 0 || first < 0 || !samples || !pederr) return MF_EINVAL;
  if (sample_stride < S.c[0].N || (S.n_sets > 1 && (sample_stride < S.c[1].N || !ctype))) return MF_EINVAL;
  if (truth && truth_stride < KMAX) return MF_EINVAL;
  if (count == 0) return MF_OK;
  if (on_device) {
    const int block = 256;
    const int64_t want = (count + block - 1) / block;
    const int grid = int(want < 152 * 64 ? want : 152 * 64);
    synth_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(*p, S, first, count, sample_stride, samples, pederr, ctype,
                                                           truth, truth_stride);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_last_error("synth_kernel launch", e);
      return MF_ECUDA;
    }
    return MF_OK;
  }
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (count < 4096) nt = 1;
  auto work = [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i)
      synth_channel(*p, S, uint64_t(first + i), samples + i * sample_stride, sample_stride, pederr + i,
                    ctype ? ctype + i : nullptr, truth ? truth + i * truth_stride : nullptr, truth_stride);
  };
  if (nt == 1) {
    work(0, count);
    return MF_OK;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (count + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = lo + chunk < count ? lo + chunk : count;
    if (lo < hi) pool.emplace_back(work, lo, hi);
  }
  for (auto& th : pool) th.join();
  return MF_OK;
}
